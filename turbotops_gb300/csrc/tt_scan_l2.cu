// tt_scan_l2.cu — instantiates the all-pairs scanner (tt_scan.cuh) for
// one metric kind; the four kinds compile in parallel.
#define TT_SCAN_IMPL
#include "tt_scan.cuh"

namespace tt {
namespace scan {
TT_SCAN_INSTANTIATE(M_L2)
}  // namespace scan
}  // namespace tt
