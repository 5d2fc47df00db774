"""TEST INFRASTRUCTURE ONLY: the CPU oracle (checker) of the front end."""
