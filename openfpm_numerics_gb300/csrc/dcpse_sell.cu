// dcpse_sell.cu -- the batched FP32 apply on a sliced ELL layout (SELL-32,
// rows sorted by length within windows of 256).
//
// The CSR apply gives a row to G lanes and reduces their partial sums by
// shuffles.  Here a row belongs to one thread: rows are grouped in slices of
// 32 (one warp) whose entries are stored entry-major, so that entry j of the
// 32 rows of a slice is one 128-byte line per stream, and no reduction is
// needed.  Within each window of 256 consecutive rows the rows are ordered
// by length (longest first) before they are cut into slices, so a slice pads
// its rows to nearly their own length; the window keeps the rows of a block
// spatially close, so the field gathers of its warps share L1 lines.
// Padding entries carry weight 0 and a column whose value the row reads
// anyway (the row itself on one set), which adds exactly nothing.  The
// per-entry arithmetic (exact differences, compensated sums for outputs of
// order >= 2) is the CSR kernel's (RowAcc).  On a renumbered layout the
// column, weight and residual streams (read once per apply) take the
// streaming (evict-first) cache hint, so that L2 keeps the outputs, which
// leave in the caller's order, until their sectors are complete.
//
// Two schedules sum the same rows in the same order: one window of 8 slices
// per block (outputs staged and stored in row order after the window's
// barrier) or warps taking slices one at a time from a counter (for layouts
// whose slices differ in length, where that barrier would idle the warps).
// Residual streams: bf16 (RK 1, the weights' FP32 rounding to 2^-32), or FP32
// (RK 2, the weight pairs, with the field in 62-bit fixed point and a
// compensated low sum: FP64-class results).
#include <cuda_bf16.h>

#include <type_traits>

#include "dcpse_internal.h"
#include "dcpse_f32_row.cuh"

namespace dcpse {
namespace {

// a load of a once-read stream, with the evict-first hint when S
template <bool S, typename T>
__device__ __forceinline__ T ld_stream(const T* p) {
    if constexpr (S)
        return __ldcs(p);
    else
        return *p;
}

constexpr int kWin = 256;            // rows per window (one block)
constexpr int kSlice = 32;           // rows per slice (one warp)
constexpr int kSlicesPerWin = kWin / kSlice;

// window w: rank its rows by length (longest first, ties in row order),
// record the row of every (slice, lane) and each slice's length x 32.  Rows
// are positions: position r holds list row perm[r] (r without perm).
__global__ void __launch_bounds__(kWin) sell_order_kernel(const int64_t* __restrict__ rowptr, int64_t n,
                                                          int64_t nwin, const int32_t* __restrict__ perm,
                                                          int32_t* __restrict__ srow, int32_t* __restrict__ slen32) {
    __shared__ int s_len[kWin];
    for (int64_t w = blockIdx.x; w < nwin; w += gridDim.x) {
        const int t = threadIdx.x;
        const int64_t r = w * kWin + t;
        const int64_t lr = (r < n && perm) ? (int64_t)perm[r] : r;
        const int len = r < n ? (int)(rowptr[lr + 1] - rowptr[lr]) : -1;
        s_len[t] = len;
        __syncthreads();
        int rank = 0;
        for (int j = 0; j < kWin; ++j) {
            const int lj = s_len[j];
            rank += (lj > len) | ((lj == len) & (j < t));
        }
        srow[w * kWin + rank] = r < n ? (int32_t)r : -1;
        // the first row of a slice is its longest
        if ((rank & (kSlice - 1)) == 0) slen32[w * kSlicesPerWin + rank / kSlice] = (len > 0 ? len : 0) * kSlice;
        __syncthreads();
    }
}

// Column of a padding entry: the row itself on one particle set (its
// difference is exactly 0), the row's first neighbour on two sets (the row
// index need not be a support index; the row reads that value anyway), 0
// for an empty row or a lane past the last row.
__device__ __forceinline__ int32_t pad_column(int one_set, int32_t row, int64_t k, const int32_t* __restrict__ cols,
                                              int64_t rb) {
    if (row < 0) return 0;
    if (one_set) return row;
    return k > 0 ? cols[rb] : 0;
}

// warp per slice: copy the CSR entries of its 32 rows into the slice,
// entry-major, 32 entries at a time through a [32][33] shared-memory block
// per warp: each row's 32 entries are read with one coalesced load, each
// entry of the 32 rows is written with one coalesced store.  Streams: -1 the
// columns, [0, nout) the weights, [nout, 2 nout) the bf16 residuals.
__global__ void __launch_bounds__(256) sell_fill_kernel(const int64_t* __restrict__ rowptr,
                                                        const int32_t* __restrict__ cols,
                                                        const float* __restrict__ w, int64_t ws, int nout,
                                                        int64_t nslices, const int32_t* __restrict__ srow,
                                                        const int64_t* __restrict__ off, int64_t total, int one_set,
                                                        int32_t* __restrict__ scols, float* __restrict__ sw,
                                                        const uint16_t* __restrict__ r16, uint16_t* __restrict__ sr16,
                                                        int st_begin, int st_end, const int32_t* __restrict__ perm,
                                                        const int32_t* __restrict__ inv) {
    __shared__ uint32_t tiles[8][32 * 33];
    const int lane = threadIdx.x & 31;
    uint32_t* tile = tiles[threadIdx.x >> 5];
    const int64_t warp0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t s = warp0; s < nslices; s += nwarps) {
        const int32_t myrow = srow[s * kSlice + lane];  // position
        const int32_t lrow = (myrow >= 0 && perm) ? perm[myrow] : myrow;
        const int64_t b = off[s];
        const int L = (int)((off[s + 1] - b) / kSlice);
        const int64_t myrb = lrow >= 0 ? rowptr[lrow] : 0;
        const int myk = lrow >= 0 ? (int)(rowptr[lrow + 1] - myrb) : 0;
        // one set: the position itself; two sets are never permuted
        const uint32_t mypad = (uint32_t)pad_column(one_set, myrow, myk, cols, myrb);
        for (int st = st_begin; st < st_end; ++st) {
            for (int j0 = 0; j0 < L; j0 += 32) {
                for (int r = 0; r < kSlice; ++r) {
                    const int64_t rb = __shfl_sync(0xffffffffu, myrb, r);
                    const int k = __shfl_sync(0xffffffffu, myk, r);
                    const int j = j0 + lane;
                    if (j < k)
                        tile[lane * 33 + r] = st < 0      ? (uint32_t)(inv ? inv[cols[rb + j]] : cols[rb + j])
                                              : st < nout ? __float_as_uint(w[(int64_t)st * ws + rb + j])
                                                          : (uint32_t)r16[(int64_t)(st - nout) * ws + rb + j];
                }
                __syncwarp();
                const int jn = min(32, L - j0);
                for (int jj = 0; jj < jn; ++jj) {
                    const int j = j0 + jj;
                    const int64_t idx = b + (int64_t)j * kSlice + lane;
                    const bool ok = j < myk;
                    const uint32_t v = tile[jj * 33 + lane];
                    if (st < 0)
                        scols[idx] = ok ? (int32_t)v : (int32_t)mypad;
                    else if (st < nout)
                        sw[(int64_t)st * total + idx] = ok ? __uint_as_float(v) : 0.0f;
                    else
                        sr16[(int64_t)(st - nout) * total + idx] = ok ? (uint16_t)v : (uint16_t)0;
                }
                __syncwarp();
            }
        }
    }
}

// FP64 weights on the same slices: warp per slice, 16 entries at a time
// through a [16][33] block of doubles per warp (coalesced reads and writes)
__global__ void __launch_bounds__(256) sell_fill64_kernel(const int64_t* __restrict__ rowptr,
                                                          const double* __restrict__ w, int64_t ws, int nout,
                                                          int64_t nslices, const int32_t* __restrict__ srow,
                                                          const int64_t* __restrict__ off, int64_t total,
                                                          double* __restrict__ sw, const int32_t* __restrict__ perm) {
    __shared__ double tiles[8][16 * 33];
    const int lane = threadIdx.x & 31;
    double* tile = tiles[threadIdx.x >> 5];
    const int64_t warp0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t s = warp0; s < nslices; s += nwarps) {
        const int32_t myrow = srow[s * kSlice + lane];
        const int32_t lrow = (myrow >= 0 && perm) ? perm[myrow] : myrow;
        const int64_t b = off[s];
        const int L = (int)((off[s + 1] - b) / kSlice);
        const int64_t myrb = lrow >= 0 ? rowptr[lrow] : 0;
        const int myk = lrow >= 0 ? (int)(rowptr[lrow + 1] - myrb) : 0;
        for (int o = 0; o < nout; ++o) {
            for (int j0 = 0; j0 < L; j0 += 16) {
                // lanes 0-15 read entries of row r, lanes 16-31 of row r + 1
                for (int r = 0; r < kSlice; r += 2) {
                    const int rr = r + (lane >> 4);
                    const int64_t rb = __shfl_sync(0xffffffffu, myrb, rr);
                    const int k = __shfl_sync(0xffffffffu, myk, rr);
                    const int j = j0 + (lane & 15);
                    if (j < k) tile[(lane & 15) * 33 + rr] = w[(int64_t)o * ws + rb + j];
                }
                __syncwarp();
                const int jn = min(16, L - j0);
                for (int jj = 0; jj < jn; ++jj) {
                    const int j = j0 + jj;
                    sw[(int64_t)o * total + b + (int64_t)j * kSlice + lane] = j < myk ? tile[jj * 33 + lane] : 0.0;
                }
                __syncwarp();
            }
        }
    }
}

// FP64 batched apply on the slices: a row per thread, summed weights, the
// difference form acc_o += w_o (f_q - f_p) with fused multiply-adds (the
// CSR FP64 kernel's arithmetic without its cross-lane reduction)
template <int NO, bool STREAM>
__global__ void __launch_bounds__(256) apply_sell64_kernel(Sell64Args a) {
    __shared__ double tile[NO][kWin];
    const int lane = threadIdx.x & 31;
    constexpr int U = 2;  // 38 registers at four outputs: six CTAs per SM
    for (int64_t win = blockIdx.x; win < a.nwin; win += gridDim.x) {
        const int64_t s = win * kSlicesPerWin + (threadIdx.x >> 5);
        const int32_t row = a.srow[s * kSlice + lane];
        const int64_t b = a.off[s];
        const int L = (int)((a.off[s + 1] - b) / kSlice);
        const double fp = (row >= 0 && !a.no_self) ? a.f[(int64_t)row * a.fs] : 0.0;
        double acc[NO];
#pragma unroll
        for (int o = 0; o < NO; ++o) acc[o] = 0.0;
        const int32_t* __restrict__ c = a.cols + b + lane;
        const double* __restrict__ w = a.w + b + lane;
        for (int j0 = 0; j0 < L; j0 += U) {
            int32_t q[U];
            double wv[U][NO], fq[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int j = j0 + u;
                const bool ok = j < L;
                q[u] = ok ? ld_stream<STREAM>(c + (int64_t)j * kSlice) : 0;
#pragma unroll
                for (int o = 0; o < NO; ++o)
                    wv[u][o] = ok ? ld_stream<STREAM>(w + (int64_t)o * a.total + (int64_t)j * kSlice) : 0.0;
            }
#pragma unroll
            for (int u = 0; u < U; ++u) fq[u] = j0 + u < L ? a.f[(int64_t)q[u] * a.fs] : fp;
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const double d = fq[u] - fp;
#pragma unroll
                for (int o = 0; o < NO; ++o) acc[o] = fma(wv[u][o], d, acc[o]);
            }
        }
        if (row >= 0) {
#pragma unroll
            for (int o = 0; o < NO; ++o) tile[o][row - win * kWin] = acc[o];
        }
        __syncthreads();
        const int64_t r = win * kWin + threadIdx.x;
        if (r < a.n) {
            const int64_t lr = a.perm ? (int64_t)a.perm[r] : r;
#pragma unroll
            for (int o = 0; o < NO; ++o) a.out[(int64_t)o * a.oos + lr * a.ors] = tile[o][threadIdx.x];
        }
        __syncthreads();
    }
}

// Whether a slice loads its column stream one chunk ahead (U more registers
// a thread): wherever ptxas reports no spills under the kernels' launch
// bounds, i.e. not for one output, not for 6 outputs of plain FP32 or weight
// pairs, and in the bound pass only with bf16 residual streams (but 6
// outputs) or plain FP32 with 2-4 or 7 outputs.  Plain FP32 with 4 outputs
// takes it at four blocks per SM (56 registers; 128^3 lattice 0.591 -> 0.577
// ms against five blocks without it).  Measured at 128^3 (window schedule):
// bf16 residual streams 1.090 -> 0.880 ms, weight pairs 1.168 -> 1.035 ms;
// graded 2D cloud, FP32: 0.150 -> 0.146 ms (warp schedule).
template <int NO, int RK, bool BOUND>
constexpr bool kPipeColumns =
    NO != 1 && (BOUND ? (RK == 1 ? NO != 6 : (NO <= 4 || NO == 7)) : (RK == 1 || (NO != 6)));

// One slice: lane `lane` sums row `row` (a position, -1 past the last row)
// over the slice's entries into acc (and, with BOUND, its weight-rounding
// bound into bs).
template <int NO, int U, int RK, bool BOUND, bool STREAM>
__device__ __forceinline__ void sell_slice(const SellArgs& a, int64_t s, int lane, int32_t row,
                                           RowAcc<NO, (RK != 0), (RK == 2)>& acc, float (&bs)[NO]) {
    const int64_t b = a.off[s];
    const int L = (int)((a.off[s + 1] - b) / kSlice);
    // the field: float pairs, or (weight pairs) fixed point
    using FT = typename std::conditional<RK == 2, long long, float2>::type;
    const FT* __restrict__ fld = RK == 2 ? reinterpret_cast<const FT*>(a.fx) : reinterpret_cast<const FT*>(a.f2);
    const FT fp = (row >= 0 && !a.no_self) ? fld[row] : FT{};
    acc.init();
#pragma unroll
    for (int o = 0; o < NO; ++o) bs[o] = 0.0f;
    const int32_t* __restrict__ c = a.cols + b + lane;
    const float* __restrict__ w = a.w + b + lane;
    // residual streams: bf16 (RK 1) or FP32 (RK 2, the weight pairs)
    const __nv_bfloat16* __restrict__ rr = RK == 1 ? a.r + b + lane : nullptr;
    const float* __restrict__ rf = RK == 2 ? a.r32 + b + lane : nullptr;
    // with kPipeColumns the column stream runs one chunk ahead: a chunk's
    // field gathers are issued beside its weight loads, not after a round
    // trip for its columns
    constexpr bool PIPE = kPipeColumns<NO, RK, BOUND>;
    int32_t qn[PIPE ? U : 1];
    if constexpr (PIPE) {
#pragma unroll
        for (int u = 0; u < U; ++u) qn[u] = u < L ? ld_stream<STREAM>(c + (int64_t)u * kSlice) : 0;
    }
    for (int j0 = 0; j0 < L; j0 += U) {
        int32_t q[U];
        float wv[U][NO], rv[U][NO];
        // entries past the slice end take the row's own value (a zero
        // difference; zero for interpolation) with weight 0: no gather
        FT fq[U];
        // the chunk's weight (and residual) streams
        auto load_weights = [&] {
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int j = j0 + u;
                const bool ok = j < L;
                if constexpr (!PIPE) q[u] = ok ? ld_stream<STREAM>(c + (int64_t)j * kSlice) : 0;
#pragma unroll
                for (int o = 0; o < NO; ++o) {
                    wv[u][o] = ok ? ld_stream<STREAM>(w + (int64_t)o * a.total + (int64_t)j * kSlice) : 0.0f;
                    if (RK == 1)
                        rv[u][o] = ok ? __bfloat162float(
                                            ld_stream<STREAM>(rr + (int64_t)o * a.total + (int64_t)j * kSlice))
                                      : 0.0f;
                    else if (RK == 2)
                        rv[u][o] = ok ? ld_stream<STREAM>(rf + (int64_t)o * a.total + (int64_t)j * kSlice) : 0.0f;
                    else
                        rv[u][o] = 0.0f;
                }
            }
        };
        if constexpr (PIPE) {
            // gathers of this chunk, columns of the next, then the weights
#pragma unroll
            for (int u = 0; u < U; ++u) fq[u] = j0 + u < L ? fld[qn[u]] : fp;
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int j = j0 + U + u;
                qn[u] = j < L ? ld_stream<STREAM>(c + (int64_t)j * kSlice) : 0;
            }
            load_weights();
        } else {
            // columns and weights, then the gathers
            load_weights();
#pragma unroll
            for (int u = 0; u < U; ++u) fq[u] = j0 + u < L ? fld[q[u]] : fp;
        }
#pragma unroll
        for (int u = 0; u < U; ++u) acc.add(wv[u], rv[u], fq[u], fp, a.comp);
        if constexpr (BOUND) {
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const float df = fabsf(fq[u].x - fp.x);
#pragma unroll
                for (int o = 0; o < NO; ++o) bs[o] = fmaf(fabsf(wv[u][o]), df, bs[o]);
            }
        }
    }
}

// output o of a summed row (fixed point: the sums are in units of
// 2^(64 - shift))
template <int NO, int RK>
__device__ __forceinline__ double sell_value(const RowAcc<NO, (RK != 0), (RK == 2)>& acc, int o, long long shift) {
    const double v = acc.value(o);
    if constexpr (RK == 2)
        return shift == kFixedNonFinite ? __longlong_as_double(0x7ff8000000000000ll) : ldexp(v, (int)(64 - shift));
    return v;
}

// thread per row; block = one window of 8 slices (five blocks per SM fit the
// registers without spills up to three outputs, four up to six, three above).
// BOUND: also the weight-rounding bound of every output of every row,
// B_o = sum_q |w_o,pq| |f_q - f_p| (FP32), stored to bnd[o * n + r], and the
// largest |output| of the call per output, atomically maxed into maxabs[o]
// (float bits; the values are >= 0, so unsigned order is float order).
template <int NO, int U, int RK, bool BOUND, bool STREAM>
__global__ void __launch_bounds__(256, (NO <= 3 && RK == 0 && !BOUND ? 5 : (NO <= 6 ? 4 : 3)))
    apply_sell_kernel(SellArgs a) {
    // the window's outputs, staged so that they leave in row order (rows of a
    // slice are permuted; scattered 8-byte stores are slow, above all into
    // host memory over NVLink-C2C)
    __shared__ double tile[NO][kWin];
    __shared__ float btile[BOUND ? NO : 1][BOUND ? kWin : 1];
    __shared__ unsigned wmax[BOUND ? NO : 1][BOUND ? kSlicesPerWin : 1];
    const int lane = threadIdx.x & 31;
    const long long shift = RK == 2 ? a.fx_meta[1] : 0;
    for (int64_t win = a.w0 + blockIdx.x; win < a.w1; win += gridDim.x) {
        const int64_t s = win * kSlicesPerWin + (threadIdx.x >> 5);  // < nslices: windows hold 8 slices
        const int32_t row = a.srow[s * kSlice + lane];
        RowAcc<NO, (RK != 0), (RK == 2)> acc;
        float bs[NO];
        sell_slice<NO, U, RK, BOUND, STREAM>(a, s, lane, row, acc, bs);
        if (row >= 0) {
#pragma unroll
            for (int o = 0; o < NO; ++o) {
                tile[o][row - win * kWin] = sell_value<NO, RK>(acc, o, shift);
                if (BOUND) btile[o][row - win * kWin] = bs[o];
            }
        }
        if (BOUND) {
            // largest |output| of the window: warp maxima, then one thread
            // per output updates the call's maximum (skipped when the stored
            // maximum is already larger)
#pragma unroll
            for (int o = 0; o < NO; ++o) {
                const unsigned v = row >= 0 ? __float_as_uint(fabsf((float)acc.value(o))) : 0u;
                const unsigned m = __reduce_max_sync(0xffffffffu, v);
                if (lane == 0) wmax[o][threadIdx.x >> 5] = m;
            }
        }
        __syncthreads();
        const int64_t r = win * kWin + threadIdx.x;
        if (r < a.n) {
            // position r holds list row perm[r]: outputs and bounds go to it
            const int64_t lr = a.perm ? (int64_t)a.perm[r] : r;
#pragma unroll
            for (int o = 0; o < NO; ++o) {
                a.out[(int64_t)o * a.oos + lr * a.ors] = tile[o][threadIdx.x];
                if (BOUND) a.bnd[(int64_t)o * a.n + lr] = btile[o][threadIdx.x];
            }
        }
        if (BOUND && threadIdx.x < NO) {
            const int o = threadIdx.x;
            unsigned m = wmax[o][0];
#pragma unroll
            for (int i = 1; i < kSlicesPerWin; ++i) m = max(m, wmax[o][i]);
            if (m > __ldcg(&a.maxabs[o])) atomicMax(&a.maxabs[o], m);
        }
        __syncthreads();  // the next window rewrites the tile
    }
}

// The same sums with warps scheduled one slice at a time: each warp takes the
// next slice of [w0 * 8, w1 * 8) from a counter (zeroed before the launch;
// the next index is fetched while the current slice is summed) and stores its
// rows' outputs directly.  Slices of a window differ in length (rows sorted
// by length within it), so the tile kernel's warps wait at the window's
// barrier for its longest slice; here no warp waits for another.  The
// stores scatter within the window's 256 rows: device-memory outputs only
// (L2 completes their sectors).  BOUND: the bounds are stored per row and
// each warp maxes |output| into maxabs (one atomic per output and slice,
// skipped when the stored maximum is already larger).
// (launch bounds as the tile kernel's, but three blocks per SM for the bound
// pass of six outputs, which spills at four)
template <int NO, int U, int RK, bool BOUND, bool STREAM>
__global__ void __launch_bounds__(256, (NO <= 3 && RK == 0 && !BOUND ? 5 : (NO < 6 || (NO == 6 && !BOUND) ? 4 : 3)))
    apply_sell_dyn_kernel(SellArgs a) {
    const int lane = threadIdx.x & 31;
    const long long shift = RK == 2 ? a.fx_meta[1] : 0;
    const int64_t s0 = a.w0 * kSlicesPerWin, s1 = a.w1 * kSlicesPerWin;
    unsigned next = lane == 0 ? atomicAdd(a.counter, 1u) : 0u;
    int64_t s = s0 + __shfl_sync(0xffffffffu, next, 0);
    while (s < s1) {
        next = lane == 0 ? atomicAdd(a.counter, 1u) : 0u;
        const int32_t row = a.srow[s * kSlice + lane];
        RowAcc<NO, (RK != 0), (RK == 2)> acc;
        float bs[NO];
        sell_slice<NO, U, RK, BOUND, STREAM>(a, s, lane, row, acc, bs);
        if (row >= 0) {
            const int64_t lr = a.perm ? (int64_t)a.perm[row] : row;
#pragma unroll
            for (int o = 0; o < NO; ++o) {
                a.out[(int64_t)o * a.oos + lr * a.ors] = sell_value<NO, RK>(acc, o, shift);
                if (BOUND) a.bnd[(int64_t)o * a.n + lr] = bs[o];
            }
        }
        if constexpr (BOUND) {
#pragma unroll
            for (int o = 0; o < NO; ++o) {
                const unsigned v = row >= 0 ? __float_as_uint(fabsf((float)acc.value(o))) : 0u;
                const unsigned m = __reduce_max_sync(0xffffffffu, v);
                if (lane == 0 && m > __ldcg(&a.maxabs[o])) atomicMax(&a.maxabs[o], m);
            }
        }
        s = s0 + __shfl_sync(0xffffffffu, next, 0);
    }
}

// Sums over all entries (p, q) of |q - p| (the list's own numbering) and of
// |inv[q] - inv[p]| (the cell order's): one warp per row, one atomic pair
// per warp.
__global__ void __launch_bounds__(256) locality_kernel(const int64_t* __restrict__ rowptr,
                                                       const int32_t* __restrict__ cols, int64_t n,
                                                       const int32_t* __restrict__ inv,
                                                       unsigned long long* __restrict__ sums) {
    const int lane = threadIdx.x & 31;
    unsigned long long a0 = 0, a1 = 0;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t p = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; p < n; p += nw) {
        const int64_t ip = inv[p];
        for (int64_t j = rowptr[p] + lane; j < rowptr[p + 1]; j += 32) {
            const int64_t q = cols[j];
            a0 += (unsigned long long)(q > p ? q - p : p - q);
            const int64_t iq = inv[q];
            a1 += (unsigned long long)(iq > ip ? iq - ip : ip - iq);
        }
    }
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) {
        a0 += __shfl_xor_sync(0xffffffffu, a0, m);
        a1 += __shfl_xor_sync(0xffffffffu, a1, m);
    }
    if (lane == 0) {
        atomicAdd(&sums[0], a0);
        atomicAdd(&sums[1], a1);
    }
}

// (hi, lo) float pair of f[i] stored at position inv[i]
__global__ void split_perm_kernel(const double* __restrict__ f, int64_t n, const int32_t* __restrict__ inv,
                                  float2* __restrict__ f2) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double v = f[i];
        const float hi = (float)v;
        f2[inv[i]] = make_float2(hi, (float)(v - (double)hi));
    }
}

// max |f| as the bits of a non-negative double (their unsigned order is the
// values' order; a NaN or an infinity compares above every finite value)
__global__ void __launch_bounds__(256) fixed_max_kernel(const double* __restrict__ f, int64_t n,
                                                        unsigned long long* __restrict__ mx) {
    unsigned long long m = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        m = max(m, (unsigned long long)__double_as_longlong(f[i]) & 0x7fffffffffffffffull);
#pragma unroll
    for (int k = 16; k > 0; k >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, k));
    __shared__ unsigned long long wm[8];
    if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < (int)(blockDim.x >> 5); ++k) m = max(m, wm[k]);
        if (m) atomicMax(mx, m);
    }
}

// fx[inv[i]] = f[i] 2^shift rounded to the nearest integer, shift = 62 - e
// with max |f| < 2^e (frexp), so |fx| < 2^62: every |f| >= 2^-9 max |f| is
// held exactly (its ulp is at least the quantum), smaller ones to 2^-62 max |f|
__global__ void __launch_bounds__(256) fixed_quant_kernel(const double* __restrict__ f, int64_t n,
                                                          const int32_t* __restrict__ inv,
                                                          long long* __restrict__ fx, long long* meta) {
    const unsigned long long mb = (unsigned long long)meta[0];
    const bool finite = mb < 0x7ff0000000000000ull;
    int e = 0;
    if (finite) frexp(__longlong_as_double((long long)mb), &e);
    const int shift = 62 - e;
    if (blockIdx.x == 0 && threadIdx.x == 0) meta[1] = finite ? shift : kFixedNonFinite;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const long long v = finite ? __double2ll_rn(ldexp(f[i], shift)) : 0;
        fx[inv ? (int64_t)inv[i] : i] = v;
    }
}

// f[i] stored at position inv[i] (FP64)
__global__ void permute_f64_kernel(const double* __restrict__ f, int64_t n, const int32_t* __restrict__ inv,
                                   double* __restrict__ g) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        g[inv[i]] = f[i];
}

__global__ void invert_kernel(const int32_t* __restrict__ perm, int64_t n, int32_t* __restrict__ inv) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        inv[perm[i]] = (int32_t)i;
}

int grid_for(int64_t n) {
    const int64_t g = (n + 255) / 256;
    const int64_t cap = (int64_t)num_sms() * 8;
    return (int)std::max<int64_t>(1, std::min(g, cap));
}

}  // namespace

cudaError_t sell_locality(const int64_t* rowptr, const int32_t* cols, int64_t n, const int32_t* inv,
                          unsigned long long* d_sums, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(d_sums, 0, 2 * sizeof(unsigned long long), s);
    if (e != cudaSuccess || n == 0) return e;
    locality_kernel<<<grid_for(n * 32), 256, 0, s>>>(rowptr, cols, n, inv, d_sums);
    return cudaGetLastError();
}

cudaError_t invert_perm(const int32_t* perm, int64_t n, int32_t* inv, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    invert_kernel<<<grid_for(n), 256, 0, s>>>(perm, n, inv);
    return cudaGetLastError();
}

cudaError_t split_f64_perm(const double* f, int64_t n, const int32_t* inv, float2* f2, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    split_perm_kernel<<<grid_for(n), 256, 0, s>>>(f, n, inv, f2);
    return cudaGetLastError();
}

cudaError_t fixed_field(const double* f, int64_t n, const int32_t* inv, long long* fx, long long* meta,
                        cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(meta, 0, 2 * sizeof(long long), s);
    if (e != cudaSuccess || n == 0) return e;
    const int grid = grid_for(n);
    fixed_max_kernel<<<grid, 256, 0, s>>>(f, n, reinterpret_cast<unsigned long long*>(meta));
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    fixed_quant_kernel<<<grid, 256, 0, s>>>(f, n, inv, fx, meta);
    return cudaGetLastError();
}

cudaError_t permute_f64(const double* f, int64_t n, const int32_t* inv, double* g, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    permute_f64_kernel<<<grid_for(n), 256, 0, s>>>(f, n, inv, g);
    return cudaGetLastError();
}

int64_t sell_slices(int64_t n) { return ((n + kWin - 1) / kWin) * kSlicesPerWin; }

cudaError_t sell_order(const int64_t* rowptr, int64_t n, int32_t* srow, int32_t* slen32, int64_t* off,
                       int64_t* scan_tmp, cudaStream_t s, const int32_t* perm) {
    const int64_t nwin = (n + kWin - 1) / kWin;
    if (nwin == 0) return cudaSuccess;
    const int grid = (int)std::min<int64_t>(nwin, (int64_t)num_sms() * 8);
    sell_order_kernel<<<grid, kWin, 0, s>>>(rowptr, n, nwin, perm, srow, slen32);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return exclusive_scan_i32(slen32, nwin * kSlicesPerWin, off, scan_tmp, s);
}

cudaError_t sell_fill(const int64_t* rowptr, const int32_t* cols, const float* w, const void* r16, int64_t ws,
                      int nout, int64_t n, int one_set, const int32_t* srow, const int64_t* off, int64_t total,
                      int32_t* scols, float* sw, void* sr16, cudaStream_t s, const int32_t* perm,
                      const int32_t* inv) {
    const int64_t ns = sell_slices(n);
    if (ns == 0) return cudaSuccess;
    // the columns when scols is given, the weights when sw is, the residual
    // streams when sr16 is (consecutive stream ranges)
    const int st_begin = scols ? -1 : (sw ? 0 : nout);
    const int st_end = sr16 ? 2 * nout : (sw ? nout : 0);
    if (st_end <= st_begin) return cudaSuccess;
    const int grid = (int)std::min<int64_t>((ns + 7) / 8, (int64_t)num_sms() * 6);
    sell_fill_kernel<<<grid, 256, 0, s>>>(rowptr, cols, w, ws, nout, ns, srow, off, total, one_set, scols, sw,
                                          static_cast<const uint16_t*>(r16), static_cast<uint16_t*>(sr16), st_begin,
                                          st_end, perm, inv);
    return cudaGetLastError();
}

cudaError_t sell_fill64(const int64_t* rowptr, const double* w, int64_t ws, int nout, int64_t n,
                        const int32_t* srow, const int64_t* off, int64_t total, double* sw, cudaStream_t s,
                        const int32_t* perm) {
    const int64_t ns = sell_slices(n);
    if (ns == 0) return cudaSuccess;
    const int grid = (int)std::min<int64_t>((ns + 7) / 8, (int64_t)num_sms() * 6);
    sell_fill64_kernel<<<grid, 256, 0, s>>>(rowptr, w, ws, nout, ns, srow, off, total, sw, perm);
    return cudaGetLastError();
}

cudaError_t apply_sell64(const Sell64Args& a, int nout, cudaStream_t s) {
    if (a.nwin == 0) return cudaSuccess;
    if (a.nwin > 0x7fffffff) return cudaErrorInvalidValue;
    switch (nout) {
#define DCPSE_SELL64_CASE(NO)                                                     \
    case NO:                                                                      \
        if (a.stream)                                                             \
            apply_sell64_kernel<NO, true><<<(unsigned)a.nwin, 256, 0, s>>>(a);    \
        else                                                                      \
            apply_sell64_kernel<NO, false><<<(unsigned)a.nwin, 256, 0, s>>>(a);   \
        break;
        DCPSE_SELL64_CASE(1)
        DCPSE_SELL64_CASE(2)
        DCPSE_SELL64_CASE(3)
        DCPSE_SELL64_CASE(4)
        DCPSE_SELL64_CASE(5)
        DCPSE_SELL64_CASE(6)
        DCPSE_SELL64_CASE(7)
        DCPSE_SELL64_CASE(8)
#undef DCPSE_SELL64_CASE
        default:
            return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

namespace {
// blocks of the warp-scheduled kernel: as many as fit on the GPU at once,
// fewer when the range has fewer slices than their warps
template <auto K>
unsigned dyn_grid(int64_t slices) {
    // blocks per SM: a property of the kernel and the architecture (the SM
    // count is looked up per device); a wrong value would only size the grid
    static const int per_sm = [] {
        int b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, K, 256, 0) != cudaSuccess || b < 1) b = 1;
        return b;
    }();
    const int64_t full = (int64_t)per_sm * num_sms();
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>(full, (slices + 7) / 8));
}

template <int NO, bool ST>
void launch_sell(const SellArgs& a, unsigned grid, cudaStream_t s) {
    constexpr int UR = NO == 1 ? 8 : (NO <= 2 ? 4 : 2);  // with the residual streams
    constexpr int U = NO == 1 ? 8 : 4;
    if (a.counter) {
        const int64_t slices = (a.w1 - a.w0) * kSlicesPerWin;
#define DCPSE_DYN(UU, RK, B) \
    apply_sell_dyn_kernel<NO, UU, RK, B, ST><<<dyn_grid<apply_sell_dyn_kernel<NO, UU, RK, B, ST>>(slices), 256, 0, s>>>(a)
        if (a.r32)
            DCPSE_DYN(UR, 2, false);
        else if (a.r && a.bnd)
            DCPSE_DYN(UR, 1, true);
        else if (a.r)
            DCPSE_DYN(UR, 1, false);
        else if (a.bnd)
            DCPSE_DYN(U, 0, true);
        else
            DCPSE_DYN(U, 0, false);
#undef DCPSE_DYN
        return;
    }
    if (a.r32)
        apply_sell_kernel<NO, UR, 2, false, ST><<<grid, 256, 0, s>>>(a);
    else if (a.r && a.bnd)
        apply_sell_kernel<NO, UR, 1, true, ST><<<grid, 256, 0, s>>>(a);
    else if (a.r)
        apply_sell_kernel<NO, UR, 1, false, ST><<<grid, 256, 0, s>>>(a);
    else if (a.bnd)
        apply_sell_kernel<NO, U, 0, true, ST><<<grid, 256, 0, s>>>(a);
    else
        apply_sell_kernel<NO, U, 0, false, ST><<<grid, 256, 0, s>>>(a);
}
}  // namespace

cudaError_t apply_sell(const SellArgs& a, int nout, cudaStream_t s) {
    if (a.w1 <= a.w0) return cudaSuccess;
    if (a.counter) {
        cudaError_t e = cudaMemsetAsync(a.counter, 0, sizeof(unsigned), s);
        if (e != cudaSuccess) return e;
    }
    // one block per window: the block scheduler balances the windows
    const int64_t grid = a.w1 - a.w0;
    if (grid > 0x7fffffff) return cudaErrorInvalidValue;
    // entries in flight per thread: 8 for one output (a row per thread walks
    // its whole row; one weight stream leaves the registers), 4 above, 2 with
    // the residual streams beyond two outputs (no register spills)
    switch (nout) {
#define DCPSE_SELL_CASE(NO)                                                                      \
    case NO:                                                                                     \
        if (a.stream)                                                                            \
            launch_sell<NO, true>(a, (unsigned)grid, s);                                         \
        else                                                                                     \
            launch_sell<NO, false>(a, (unsigned)grid, s);                                        \
        break;
        DCPSE_SELL_CASE(1)
        DCPSE_SELL_CASE(2)
        DCPSE_SELL_CASE(3)
        DCPSE_SELL_CASE(4)
        DCPSE_SELL_CASE(5)
        DCPSE_SELL_CASE(6)
        DCPSE_SELL_CASE(7)
        DCPSE_SELL_CASE(8)
#undef DCPSE_SELL_CASE
        default:
            return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace dcpse
