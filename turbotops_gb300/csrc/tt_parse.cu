// tt_parse.cu — read_text_points (src/turbotops.cpp:126-155) on the device.
//
// The reference reads a text file line by line (std::getline: lines end at
// '\n'), cuts each line at its first '#', turns ',', '\t' and ';' into
// spaces, splits it into tokens at the C locale's white space (' ', '\t',
// '\n', '\v', '\f', '\r') and converts every token with std::strtof, which
// must consume all of it ("bad coordinate '<token>'" otherwise). Lines
// without tokens are skipped; the first line with tokens sets the dimension
// and every later one must match it ("inconsistent row length at point N",
// N the 0-based index of the offending point). Errors are reported in file
// order: the first line holding a bad token or a wrong count decides, a bad
// token before the count check of its own line.
//
// Here the file's bytes go to the device in one copy; one pass finds the
// lines, one counts each line's tokens (a warp a line), and one converts
// them (a warp a line, a lane a token) into the n x dim matrix. Decimal
// tokens ([sign] digits [. digits] [e|E [sign] digits]) and "inf" /
// "infinity" are converted on the device, correctly rounded as strtof
// rounds them (nearest, ties to even; the conversion below is exact
// integer arithmetic). Every other token (hexadecimal floats, NaN spellings,
// anything strtof may still accept or reject) and the rare decimal whose
// rounding its first 19 significant digits cannot decide go back to the host,
// which calls the host C library's strtof on the token itself, as the
// reference does. The host also reports the first error.
#include <algorithm>
#include <cerrno>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "tt_internal.cuh"

namespace tt {
namespace {

// A token handed to the host: where it is and where its value goes.
struct HostTok {
    u64 off;    // byte offset in the text
    u64 slot;   // output index (point * dim + column)
    u32 len;
    u32 line;
};

__device__ __forceinline__ bool is_sep(u32 c) {
    return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r' || c == ',' || c == ';';
}

// ---- exact decimal -> binary32 --------------------------------------------
// Unsigned 192-bit integers, little-endian limbs.
struct U192 {
    u64 w[3];
};

__device__ __forceinline__ int bitlen(const U192& a) {
    if (a.w[2]) return 128 + 64 - __clzll(a.w[2]);
    if (a.w[1]) return 64 + 64 - __clzll(a.w[1]);
    return a.w[0] ? 64 - __clzll(a.w[0]) : 0;
}

__device__ __forceinline__ void mul_small(U192& a, u64 m) {   // a *= m (the product fits 192 bits)
    u64 carry = 0;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const u64 lo = a.w[i] * m + carry;
        carry = __umul64hi(a.w[i], m) + (lo < carry ? 1 : 0);
        a.w[i] = lo;
    }
}

__device__ __forceinline__ U192 shl(const U192& a, int s) {   // s < 192
    U192 r{{0, 0, 0}};
    const int q = s >> 6, b = s & 63;
#pragma unroll
    for (int i = 2; i >= 0; --i) {
        const int j = i - q;
        if (j < 0) continue;
        u64 v = a.w[j] << b;
        if (b && j > 0) v |= a.w[j - 1] >> (64 - b);
        r.w[i] = v;
    }
    return r;
}

__device__ __forceinline__ bool geq(const U192& a, const U192& b) {
    if (a.w[2] != b.w[2]) return a.w[2] > b.w[2];
    if (a.w[1] != b.w[1]) return a.w[1] > b.w[1];
    return a.w[0] >= b.w[0];
}

__device__ __forceinline__ void sub(U192& a, const U192& b) {   // a -= b, a >= b
    u64 borrow = 0;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const u64 t = a.w[i] - b.w[i];
        const u64 nb = (a.w[i] < b.w[i]) | (t < borrow);
        a.w[i] = t - borrow;
        borrow = nb;
    }
}

__device__ __forceinline__ U192 pow5(int k) {   // 5^k, k <= 82 (< 2^191)
    U192 r{{1, 0, 0}};
    for (; k >= 13; k -= 13) mul_small(r, 1220703125ull);   // 5^13
    u64 m = 1;
    for (; k > 0; --k) m *= 5;
    mul_small(r, m);
    return r;
}

// Rounds to nearest, ties to even: hi_bits holds the value's leading bits,
// the float keeps hi_bits >> shift (24 bits for a normal result, fewer for a
// subnormal), sticky_below says whether anything below hi_bits is set, e is
// the binary exponent of the leading bit. Returns the float's bits
// (0x7f800000 on overflow).
__device__ __forceinline__ u32 round_bits(u64 hi_bits, int shift, bool sticky_below, int e) {
    // hi_bits >> shift is the kept part; bit shift - 1 the round bit (shift
    // may exceed 63 for values far below the smallest subnormal)
    u64 mant = shift < 64 ? hi_bits >> shift : 0;
    const bool rb = shift > 0 && shift <= 64 && ((hi_bits >> (shift - 1)) & 1u);
    const u64 below = shift <= 1 ? 0 : shift > 64 ? hi_bits : hi_bits & ((1ull << (shift - 1)) - 1);
    const bool st = sticky_below || below != 0;
    if (rb && (st || (mant & 1u))) ++mant;
    if (e >= -126) {   // normal: mant has 24 bits (or 2^24 after the carry)
        if (mant == (1ull << 24)) {
            mant >>= 1;
            ++e;
        }
        if (e > 127) return 0x7f800000u;
        return (u32(e + 127) << 23) | (u32(mant) & 0x7fffffu);
    }
    return u32(mant);   // subnormal (2^23 becomes the smallest normal: the same bits)
}

// The float32 nearest to w * 10^q (ties to even), w > 0: exact integer
// arithmetic. q >= 0: N = w 5^q, the value N 2^q. q < 0: Q = floor(w 2^s /
// 5^-q) with at least 27 bits and the remainder as a sticky bit, the value
// (Q + f) 2^(-s + q).
__device__ u32 dec_to_f32(u64 w, int q) {
    if (q >= 0) {
        if (q > 38) return 0x7f800000u;
        if (w < (1ull << 24) && q <= 10) {   // exact operands, one rounding
            float p = 1.0f;
            for (int i = 0; i < q; ++i) p *= 10.0f;   // 10^q, q <= 10: exact
            return __float_as_uint(__fmul_rn(float(w), p));
        }
        U192 n = pow5(q);
        {
            // n *= w (w < 2^64): two 32-bit halves
            U192 a = n, b = n;
            mul_small(a, w & 0xffffffffull);
            mul_small(b, w >> 32);
            b = shl(b, 32);
            u64 carry = 0;
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                const u64 s = a.w[i] + b.w[i];
                const u64 c1 = s < a.w[i];
                n.w[i] = s + carry;
                carry = c1 | (n.w[i] < s);
            }
        }
        const int L = bitlen(n);
        const int e = L - 1 + q;
        if (e > 127) return 0x7f800000u;
        if (L <= 24) return (u32(e + 127) << 23) | (u32(n.w[0] << (24 - L)) & 0x7fffffu);
        // top 64 bits of n, and whether anything below them is set
        const int drop = L > 64 ? L - 64 : 0;
        u64 top;
        bool sticky = false;
        if (drop == 0) {
            top = n.w[0];
        } else {
            const U192 t = shl(n, 192 - L);   // leading bit to bit 191
            top = t.w[2];
            sticky = t.w[1] != 0 || t.w[0] != 0;
        }
        const int tl = L - drop;   // bits in top
        return round_bits(top, tl - 24, sticky, e);
    }
    const int k = -q;
    if (k >= 65) return 0u;   // w 10^-k < 2^64 10^-65 < 2^-150: rounds to +0
    if (w < (1ull << 24) && k <= 10) {
        float p = 1.0f;
        for (int i = 0; i < k; ++i) p *= 10.0f;
        return __float_as_uint(__fdiv_rn(float(w), p));
    }
    const U192 d = pow5(k);
    const int ld = bitlen(d);
    const int lw = 64 - __clzll(w);
    const int s = max(0, 27 + ld - lw);
    U192 m = shl(U192{{w, 0, 0}}, s);
    const int qbits = bitlen(m) - ld + 1;   // the quotient has at most this many bits
    u64 Q = 0;
    for (int b = qbits - 1; b >= 0; --b) {
        const U192 db = shl(d, b);
        if (geq(m, db)) {
            sub(m, db);
            Q |= 1ull << b;
        }
    }
    const bool rem = m.w[0] | m.w[1] | m.w[2];
    const int LQ = 64 - __clzll(Q);
    const int e = LQ - 1 - s - k;
    if (e >= -126) return round_bits(Q, LQ - 24, rem, e);
    return round_bits(Q, s + k - 149, rem, e);
}

// Token at s[p..end) (end: the line's end; a separator or '#' ends it
// earlier); returns its length
// and, when the device can decide it, its value bits in *bits (status 0);
// status 1 sends it to the host.
__device__ u32 parse_token(const unsigned char* __restrict__ s, u64 p, u64 end, u32* bits, int* status) {
    u64 e = p;
    while (e < end && !is_sep(s[e]) && s[e] != '#') ++e;
    const u32 len = u32(e - p);
    *status = 1;
    u64 i = p;
    u32 sign = 0;
    if (i < e && (s[i] == '+' || s[i] == '-')) sign = s[i++] == '-' ? 0x80000000u : 0u;
    // inf / infinity, any case
    if (i < e && (s[i] | 0x20) == 'i') {
        const char* a = "infinity";
        u64 j = 0;
        while (i + j < e && j < 8 && (s[i + j] | 0x20) == a[j]) ++j;
        if ((j == 3 || j == 8) && i + j == e) {
            *bits = sign | 0x7f800000u;
            *status = 0;
        }
        return len;
    }
    u64 w = 0;
    int sig = 0;            // significant digits kept in w
    int q = 0;              // decimal exponent of w
    bool inexact = false;   // a dropped digit was not zero
    bool any = false, dot = false;
    for (; i < e; ++i) {
        const u32 c = s[i];
        if (c == '.') {
            if (dot) return len;
            dot = true;
            continue;
        }
        if (c < '0' || c > '9') break;
        any = true;
        if (sig == 0 && c == '0') {
            if (dot) --q;   // a leading zero after the point
            continue;
        }
        if (sig < 19) {
            w = w * 10 + (c - '0');
            ++sig;
            if (dot) --q;
        } else {
            if (c != '0') inexact = true;
            if (!dot) ++q;
        }
    }
    if (!any) return len;
    if (i < e) {
        if ((s[i] | 0x20) != 'e') return len;
        ++i;
        bool neg = false;
        if (i < e && (s[i] == '+' || s[i] == '-')) neg = s[i++] == '-';
        if (i >= e) return len;
        int x = 0;
        for (; i < e; ++i) {
            const u32 c = s[i];
            if (c < '0' || c > '9') return len;
            if (x < 100000) x = x * 10 + int(c - '0');
        }
        q += neg ? -x : x;
    }
    if (w == 0) {
        *bits = sign;
        *status = 0;
        return len;
    }
    q = max(-100000, min(100000, q));
    const u32 r1 = dec_to_f32(w, q);
    if (inexact) {
        // the value lies strictly between w 10^q and (w + 1) 10^q: decided
        // when both round to the same float (w + 1 <= 10^19 < 2^64)
        if (dec_to_f32(w + 1, q) != r1) return len;
    }
    *bits = sign | r1;
    *status = 0;
    return len;
}

// ---- passes -----------------------------------------------------------------
constexpr u32 kChunk = 256;   // bytes per thread when finding the lines

__global__ void k_nl_count(const unsigned char* __restrict__ s, u64 len, u32* __restrict__ cnt, u64 chunks) {
    for (u64 t = u64(blockIdx.x) * blockDim.x + threadIdx.x; t < chunks; t += u64(gridDim.x) * blockDim.x) {
        const u64 b = t * kChunk, e = min(len, b + kChunk);
        u32 c = 0;
        for (u64 i = b; i < e; ++i) c += s[i] == '\n';
        cnt[t] = c;
    }
}

// starts[0] = 0, starts[i + 1] = one past the i-th '\n'
__global__ void k_nl_fill(const unsigned char* __restrict__ s, u64 len, const u32* __restrict__ off, u64 chunks,
                          u64* __restrict__ starts) {
    for (u64 t = u64(blockIdx.x) * blockDim.x + threadIdx.x; t < chunks; t += u64(gridDim.x) * blockDim.x) {
        const u64 b = t * kChunk, e = min(len, b + kChunk);
        u64 o = u64(off[t]) + 1;
        if (t == 0) starts[0] = 0;
        for (u64 i = b; i < e; ++i)
            if (s[i] == '\n') starts[o++] = i + 1;
    }
}

// The line's token-bearing extent: [start, end) cut at its first '#'.
__device__ __forceinline__ u64 line_end(const unsigned char* __restrict__ s, const u64* __restrict__ starts,
                                        u64 line, u64 nlines, u64 len) {
    return line + 1 < nlines ? starts[line + 1] - 1 : len;
}

// Walks one line with a warp: calls f(lane_has_start, pos, chunk_end) for
// every 32-byte chunk until the line or its '#' ends; starts are bytes that
// are not separators and follow a separator or the line's start.
template <typename F>
__device__ __forceinline__ u64 walk_line(const unsigned char* __restrict__ s, u64 b, u64 e, F&& f) {
    const u32 lane = threadIdx.x & 31;
    bool prev_sep = true;   // before the line's first byte
    for (u64 c0 = b; c0 < e; c0 += 32) {
        const u64 pos = c0 + lane;
        const u32 ch = pos < e ? s[pos] : u32('\n');
        const u32 hash = __ballot_sync(0xffffffffu, ch == '#');
        const u32 valid_n = u32(e - c0 < 32 ? e - c0 : 32);
        const u32 cut = hash ? u32(__ffs(hash) - 1) : valid_n;   // bytes of this chunk in the line
        const bool sep = is_sep(ch) || lane >= cut;
        const u32 sepm = __ballot_sync(0xffffffffu, sep);
        const bool psep = lane ? (sepm >> (lane - 1)) & 1u : prev_sep;
        const bool start = !sep && psep;
        const u64 cend = hash ? c0 + cut : e;
        f(start, pos, cend);
        if (hash) return c0 + cut;
        prev_sep = (sepm >> 31) & 1u;
    }
    return e;
}

__global__ void k_line_count(const unsigned char* __restrict__ s, u64 len, const u64* __restrict__ starts, u64 nlines,
                             u32* __restrict__ cnt) {
    const u64 warps = (u64(gridDim.x) * blockDim.x) >> 5;
    for (u64 line = (u64(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; line < nlines; line += warps) {
        const u64 b = starts[line], e = line_end(s, starts, line, nlines, len);
        u32 c = 0;
        walk_line(s, b, e, [&](bool start, u64, u64) { c += __popc(__ballot_sync(0xffffffffu, start)); });
        if ((threadIdx.x & 31) == 0) cnt[line] = c;
    }
}

// The first line with tokens, and the first later line whose count differs.
__global__ void k_line_first(const u32* __restrict__ cnt, u64 nlines, unsigned long long* __restrict__ first) {
    for (u64 l = u64(blockIdx.x) * blockDim.x + threadIdx.x; l < nlines; l += u64(gridDim.x) * blockDim.x)
        if (cnt[l]) atomicMin(&first[0], (unsigned long long)l);
}
__global__ void k_line_check(const u32* __restrict__ cnt, u64 nlines, unsigned long long* __restrict__ first) {
    const u64 f = first[0];
    if (f >= nlines) return;
    const u32 dim = cnt[f];
    for (u64 l = u64(blockIdx.x) * blockDim.x + threadIdx.x; l < nlines; l += u64(gridDim.x) * blockDim.x)
        if (cnt[l] && cnt[l] != dim) atomicMin(&first[1], (unsigned long long)l);
}

__global__ void k_nonempty(const u32* __restrict__ cnt, u64 nlines, u32* __restrict__ f) {
    for (u64 l = u64(blockIdx.x) * blockDim.x + threadIdx.x; l < nlines; l += u64(gridDim.x) * blockDim.x)
        f[l] = cnt[l] != 0;
}

// Converts the tokens of lines [0, limit): lane by lane, each token start
// parses its token; the values land at point * dim + column. Line `limit`
// (the first whose count differs, if any) is only checked: the reference
// converts its tokens before it compares the count, so a bad token there is
// still the error to report; its host tokens carry slot ~0.
__global__ void k_line_parse(const unsigned char* __restrict__ s, u64 len, const u64* __restrict__ starts, u64 limit,
                             u64 nlines, const u32* __restrict__ cnt, const u32* __restrict__ point, u32 dim,
                             u32* __restrict__ out, HostTok* __restrict__ host, unsigned long long* __restrict__ nhost) {
    const u32 lane = threadIdx.x & 31;
    const u64 warps = (u64(gridDim.x) * blockDim.x) >> 5;
    const u64 last = min(limit + 1, nlines);
    for (u64 line = (u64(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; line < last; line += warps) {
        if (!cnt[line]) continue;
        const bool write = line < limit;
        const u64 b = starts[line], e = line_end(s, starts, line, nlines, len);
        const u64 base = u64(point[line]) * dim;
        u32 col = 0;
        walk_line(s, b, e, [&](bool start, u64 pos, u64 cend) {
            const u32 m = __ballot_sync(0xffffffffu, start);
            if (start) {
                const u64 slot = base + col + __popc(m & ((1u << lane) - 1u));
                u32 bits = 0;
                int st = 1;
                const u32 tl = parse_token(s, pos, cend, &bits, &st);
                if (st == 0) {
                    if (write) out[slot] = bits;
                } else {
                    const unsigned long long h = atomicAdd(nhost, 1ull);
                    host[h] = HostTok{pos, write ? slot : ~0ull, tl, u32(line)};
                }
            }
            col += __popc(m);
        });
    }
}

inline u32 grid_for(u64 work, u32 per_block) {
    const u64 g = (work + per_block - 1) / per_block;
    return u32(std::max<u64>(1, std::min<u64>(g, 64ull * kSMs)));
}

}  // namespace

// read_text_points on the device: text (host, `bytes` bytes) -> points (host,
// up to cap floats). Sets *n and *dim; throws the reference's messages (the
// row-length one without the path, which the caller prefixes).
void parse_points(tt_ctx* c, const char* text, u64 bytes, f32* pts, u64 cap, u32* n_out, u32* dim_out) {
    if (bytes >= 3 && u8(text[0]) == 0xEF && u8(text[1]) == 0xBB && u8(text[2]) == 0xBF) {
        text += 3;
        bytes -= 3;
    }
    *n_out = 0;
    *dim_out = 0;
    if (!bytes) return;
    unsigned char* s = c->arena.get<unsigned char>(S_TXT, bytes + 16);
    TT_CUDA(cudaMemcpyAsync(s, text, bytes, cudaMemcpyHostToDevice, c->stream));
    // lines
    const u64 chunks = (bytes + kChunk - 1) / kChunk;
    u32* ccnt = c->arena.get<u32>(S_TXT_CNT, chunks + 1);
    k_nl_count<<<grid_for(chunks, 256), 256, 0, c->stream>>>(s, bytes, ccnt, chunks);
    TT_LAUNCH("k_nl_count");
    u32* total = ccnt + chunks;
    scan_exclusive<u32>(c, ccnt, ccnt, chunks, total);
    u32 nl = 0;
    TT_CUDA(cudaMemcpyAsync(&nl, total, 4, cudaMemcpyDeviceToHost, c->stream));
    TT_CUDA(cudaStreamSynchronize(c->stream));
    const u64 nlines = u64(nl) + 1;
    u64* starts = c->arena.get<u64>(S_TXT_LINES, nlines + 1);
    k_nl_fill<<<grid_for(chunks, 256), 256, 0, c->stream>>>(s, bytes, ccnt, chunks, starts);
    TT_LAUNCH("k_nl_fill");
    // tokens per line, the dimension, the first inconsistent line, point indices
    u32* cnt = c->arena.get<u32>(S_TXT_TOK, 2 * nlines + 2);
    u32* point = cnt + nlines + 1;
    k_line_count<<<grid_for(nlines * 32, 256), 256, 0, c->stream>>>(s, bytes, starts, nlines, cnt);
    TT_LAUNCH("k_line_count");
    unsigned long long* first = c->arena.get<unsigned long long>(S_COUNT, 4);
    TT_CUDA(cudaMemsetAsync(first, 0xff, 2 * sizeof(unsigned long long), c->stream));
    TT_CUDA(cudaMemsetAsync(first + 2, 0, sizeof(unsigned long long), c->stream));
    k_line_first<<<grid_for(nlines, 256), 256, 0, c->stream>>>(cnt, nlines, first);
    k_line_check<<<grid_for(nlines, 256), 256, 0, c->stream>>>(cnt, nlines, first);
    k_nonempty<<<grid_for(nlines, 256), 256, 0, c->stream>>>(cnt, nlines, point);
    TT_LAUNCH("k_line_check");
    scan_exclusive<u32>(c, point, point, nlines, point + nlines);
    unsigned long long h[2];
    TT_CUDA(cudaMemcpyAsync(h, first, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    TT_CUDA(cudaStreamSynchronize(c->stream));
    c->launches += 7;
    if (h[0] >= nlines) return;   // no tokens at all
    // lines the reference converts before any count error, and that line
    const u64 limit = std::min<u64>(h[1], nlines);
    u32 dim = 0, npts = 0, bad_cnt = 0;
    TT_CUDA(cudaMemcpyAsync(&dim, cnt + h[0], 4, cudaMemcpyDeviceToHost, c->stream));
    TT_CUDA(cudaMemcpyAsync(&npts, point + limit, 4, cudaMemcpyDeviceToHost, c->stream));
    if (limit < nlines) TT_CUDA(cudaMemcpyAsync(&bad_cnt, cnt + limit, 4, cudaMemcpyDeviceToHost, c->stream));
    TT_CUDA(cudaStreamSynchronize(c->stream));
    const u64 total_vals = u64(npts) * dim;
    if (total_vals > cap) throw Error(TT_ERR_LENGTH, "gb300: points exceed the output capacity");
    // conversion
    u32* out = c->arena.get<u32>(S_OUT0, total_vals + 1);
    HostTok* host = c->arena.get<HostTok>(S_TXT_HOST, total_vals + bad_cnt + 1);
    unsigned long long* nhost = first + 2;
    k_line_parse<<<grid_for(std::min<u64>(limit + 1, nlines) * 32, 256), 256, 0, c->stream>>>(
        s, bytes, starts, limit, nlines, cnt, point, dim, out, host, nhost);
    TT_LAUNCH("k_line_parse");
    ++c->launches;
    unsigned long long nh = 0;
    TT_CUDA(cudaMemcpyAsync(&nh, nhost, 8, cudaMemcpyDeviceToHost, c->stream));
    if (total_vals) TT_CUDA(cudaMemcpyAsync(pts, out, 4 * total_vals, cudaMemcpyDeviceToHost, c->stream));
    TT_CUDA(cudaStreamSynchronize(c->stream));
    // the host's tokens, in file order: strtof over the whole token
    std::vector<HostTok> ht(nh);
    if (nh) TT_CUDA(cudaMemcpy(ht.data(), host, nh * sizeof(HostTok), cudaMemcpyDeviceToHost));
    std::sort(ht.begin(), ht.end(), [](const HostTok& a, const HostTok& b) { return a.off < b.off; });
    for (const HostTok& t : ht) {
        const std::string tok(text + t.off, t.len);
        char* end = nullptr;
        const f32 v = std::strtof(tok.c_str(), &end);
        if (!end || *end) invalid("bad coordinate '" + tok + "'");
        if (t.slot != ~0ull) pts[t.slot] = v;
    }
    if (limit < nlines) invalid("inconsistent row length at point " + std::to_string(npts));
    *n_out = npts;
    *dim_out = dim;
}

}  // namespace tt
