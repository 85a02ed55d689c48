// dcpse_neighbors.cu -- device neighbour lists (CSR) for the DC-PSE path.
//
// Replaces the reference's two support builders:
//  * CPU: openfpm VerletList getVerlet<VL_NON_SYMMETRIC|VL_SKIP_REF_PART>
//    (used by src/DCPSE/Dcpse.hpp:721 via getNNIterator);
//  * GPU: gatherSupportSize_gpu / assembleSupport_gpu with a host prefix sum
//    (src/DCPSE/SupportBuilder.cuh:14-107).
// Here every step stays on the device: cell ids, counting sort into cells,
// a count pass, a device exclusive scan, a fill pass and a per-row sort.
// The list of particle p is every q != p with |x_p - x_q|^2 < rc_p^2 in
// ascending q, so it does not depend on the cell size or on the order in
// which atomics filled the cells.
//
// The FP64 predicate is what defines the list, but GB300's FP64 pipe (2
// lanes per cycle per SM) makes it the bottleneck when it runs on every
// candidate.  Candidates are therefore first classified in FP32 from
// positions stored relative to their cell's lower corner: |d^2 - rc^2| below
// a margin of 2^-14 S^2 (S = 3 x the largest cell side; with both offsets
// from the corner below S, the FP32 error of d^2 stays below 200 u S^2 =
// 1.2e-5 S^2, u = 2^-24, corner offsets of the +-1 cells included) is decided by the
// FP64 predicate itself, as are particles outside the grid, NaN positions
// and periodic axes with fewer than three cells.  The lists are the same bit
// for bit.
#include <atomic>
#include <cstdint>
#include <cstring>

#include "dcpse_internal.h"

namespace dcpse {

namespace {

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ int64_t warp_incl_scan(int64_t v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int64_t t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// Block-wide exclusive scan (blockDim a multiple of 32); returns the
// exclusive prefix of v and the block total in *tot.
__device__ int64_t block_excl_scan(int64_t v, int64_t* tot) {
    __shared__ int64_t warp_sums[33];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int64_t inc = warp_incl_scan(v);
    if (lane == 31) warp_sums[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        int64_t w = (lane < nw) ? warp_sums[lane] : 0;
        int64_t wi = warp_incl_scan(w);
        if (lane < nw) warp_sums[lane] = wi - w;
        if (lane == 31) warp_sums[32] = wi;
    }
    __syncthreads();
    int64_t r = warp_sums[wid] + inc - v;
    *tot = warp_sums[32];
    __syncthreads();
    return r;
}

__global__ void scan_tile_sums(const int32_t* __restrict__ in, int64_t n, int64_t* __restrict__ tile_sums) {
    int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    int64_t s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i)
        if (base + i < n) s += in[base + i];
    int64_t tot;
    block_excl_scan(s, &tot);
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = tot;
}

// single block: exclusive scan of tile sums in place; tile_sums[ntiles] = total
__global__ void scan_tile_offsets(int64_t* tile_sums, int64_t ntiles) {
    __shared__ int64_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int64_t b = 0; b < ntiles; b += blockDim.x) {
        int64_t i = b + threadIdx.x;
        int64_t v = (i < ntiles) ? tile_sums[i] : 0;
        int64_t tot;
        int64_t ex = block_excl_scan(v, &tot);
        int64_t c = carry;
        if (i < ntiles) tile_sums[i] = c + ex;
        __syncthreads();
        if (threadIdx.x == 0) carry = c + tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) tile_sums[ntiles] = carry;
}

__global__ void scan_tiles(const int32_t* __restrict__ in, int64_t n, const int64_t* __restrict__ tile_off,
                           int64_t* __restrict__ out) {
    int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    int64_t v[kScanItems];
    int64_t s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        v[i] = (base + i < n) ? (int64_t)in[base + i] : 0;
        s += v[i];
    }
    int64_t tot;
    int64_t ex = block_excl_scan(s, &tot) + tile_off[blockIdx.x];
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        if (base + i < n) out[base + i] = ex;
        ex += v[i];
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) out[n] = tile_off[gridDim.x];
}

__device__ __forceinline__ unsigned long long ord_of(double x) {
    unsigned long long u = (unsigned long long)__double_as_longlong(x);
    return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}

double from_ord(unsigned long long u) {
    u = (u >> 63) ? (u & 0x7fffffffffffffffull) : ~u;
    double d;
    memcpy(&d, &u, sizeof d);
    return d;
}

__global__ void bbox_kernel(int dim, const double* __restrict__ p, int64_t n, unsigned long long* mm) {
    double lo[kMaxDim], hi[kMaxDim];
    for (int d = 0; d < kMaxDim; ++d) {
        lo[d] = INFINITY;
        hi[d] = -INFINITY;
    }
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        for (int d = 0; d < dim; ++d) {
            double x = p[i * dim + d];
            lo[d] = fmin(lo[d], x);
            hi[d] = fmax(hi[d], x);
        }
    for (int d = 0; d < dim; ++d) {
        for (int o = 16; o > 0; o >>= 1) {
            lo[d] = fmin(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], o));
            hi[d] = fmax(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], o));
        }
        if ((threadIdx.x & 31) == 0) {
            atomicMin(&mm[d], ord_of(lo[d]));
            atomicMax(&mm[kMaxDim + d], ord_of(hi[d]));
        }
    }
}

__device__ __forceinline__ int cell_coord(double x, double lo, double cs, int nc) {
    double v = floor((x - lo) / cs);
    if (!(v >= 0.0)) return 0;  // also catches NaN
    if (v >= (double)nc) return nc - 1;
    return (int)v;
}

__global__ void cell_id_kernel(int dim, const double* __restrict__ pos, int64_t n, CellGrid g,
                               int32_t* __restrict__ cell, int32_t* __restrict__ ccount) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int c[kMaxDim] = {0, 0, 0};
        for (int d = 0; d < dim; ++d) c[d] = cell_coord(pos[i * dim + d], g.lo[d], g.cs[d], g.nc[d]);
        int lin = c[0] + g.nc[0] * (c[1] + g.nc[1] * c[2]);
        cell[i] = lin;
        atomicAdd(&ccount[lin], 1);
    }
}

__global__ void cell_fill_kernel(int dim, const double* __restrict__ pos, int64_t n, const int32_t* __restrict__ cell,
                                 CellGrid g, int64_t* fill, int32_t* __restrict__ cidx, double* __restrict__ spos,
                                 float4* __restrict__ srel) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        unsigned long long slot = atomicAdd((unsigned long long*)&fill[cell[i]], 1ull);
        cidx[slot] = (int32_t)i;
        float r[kMaxDim] = {0.f, 0.f, 0.f};
        int cx = 0;
        for (int d = 0; d < dim; ++d) {
            const double x = pos[i * dim + d];
            spos[slot * dim + d] = x;
            // offset from the cell's lower corner; NaN (always the FP64
            // test) for a particle clamped into an edge cell
            const int c = cell_coord(x, g.lo[d], g.cs[d], g.nc[d]);
            if (d == 0) cx = c;
            const double rel = x - (g.lo[d] + (double)c * g.cs[d]);
            r[d] = (rel >= -0.5 * g.cs[d] && rel <= 1.5 * g.cs[d]) ? (float)rel : __int_as_float(0x7fc00000);
        }
        // w: the cell's index along axis 0, for candidates taken from a run
        // of cells along that axis
        srel[slot] = make_float4(r[0], r[1], r[2], __int_as_float(cx));
    }
}

// The stencil of one domain particle: along each axis the centre cell c and
// three slots for the cells at offsets -1, 0, +1.  A slot is dropped outside
// a non-periodic grid, or when a periodic axis of fewer than three cells
// would list a cell twice.  rpc = x_p minus the lower corner of the centre
// cell; the corner of slot t (before the periodic wrap, i.e. of the image
// next to p) is (t - 1) cell sides further.
struct Stencil {
    int c[3];
    float rpc[3];
    unsigned valid;  // bit 3 d + t: slot t of axis d is a cell
    unsigned fast;   // bit 3 d + t: |x_p - corner| <= 3 cell sides, FP32 classification allowed
};

template <int DIM>
__device__ __forceinline__ void make_stencil(const NbrArgs& a, const double* xp, Stencil& S) {
    S.valid = 0;
    S.fast = 0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        S.c[d] = 0;
        S.rpc[d] = 0.f;
        if (d >= DIM) {
            S.valid |= 1u << (3 * d + 1);
            S.fast |= 1u << (3 * d + 1);
            continue;
        }
        const int nc = a.cells.nc[d];
        const int c = cell_coord(xp[d], a.cells.lo[d], a.cells.cs[d], nc);
        S.c[d] = c;
        S.rpc[d] = (float)(xp[d] - (a.cells.lo[d] + (double)c * a.cells.cs[d]));
        int w[3];
#pragma unroll
        for (int t = 0; t < 3; ++t) {
            const int u = c + t - 1;
            bool ok = true;
            w[t] = u;
            if (a.geom.per[d]) {
                w[t] = ((u % nc) + nc) % nc;
#pragma unroll
                for (int t2 = 0; t2 < t; ++t2)
                    if (((S.valid >> (3 * d + t2)) & 1u) && w[t2] == w[t]) ok = false;
            } else if (u < 0 || u >= nc) {
                ok = false;
            }
            const double rp = xp[d] - (a.cells.lo[d] + (double)u * a.cells.cs[d]);
            if (ok) S.valid |= 1u << (3 * d + t);
            if (ok && a.fast && fabs(rp) <= 3.0 * a.cells.cs[d]) S.fast |= 1u << (3 * d + t);
        }
    }
}

// cell index of slot t around centre c along an axis (wrapped when periodic)
__device__ __forceinline__ int slot_cell(int c, int t, int nc, int per) {
    int v = c + t - 1;
    if (per) v = v < 0 ? v + nc : (v >= nc ? v - nc : v);
    return v;
}

// One warp per domain particle scans the 3^d stencil cells of the support
// cell list, 32 candidates at a time.  The per-particle set-up (cells,
// corner offsets, thresholds: FP64 work) is done one lane per particle for
// 32 particles at once and broadcast by shuffles, since a warp instruction
// costs the FP64 pipe the same whether one lane or 32 are active.
template <int DIM, bool FILL>
__global__ void __launch_bounds__(256) nbr_kernel(NbrArgs a, int32_t* __restrict__ counts, int* maxk,
                                                  const int64_t* __restrict__ rowptr, int32_t* __restrict__ tmp) {
    const int lane = threadIdx.x & 31;
    const int64_t warp0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const unsigned lt_mask = (1u << lane) - 1u;
    const unsigned full = 0xffffffffu;
    for (int64_t pb = warp0 * 32; pb < a.n_dom; pb += nwarps * 32) {
        // set-up of particle pb + lane
        float tin = 0.f, tout = 0.f;
        Stencil S;
        {
            double x[3] = {0.0, 0.0, 0.0};
            const int64_t pl = pb + lane;
            if (pl < a.n_dom) {
#pragma unroll
                for (int d = 0; d < DIM; ++d) x[d] = a.pd[pl * DIM + d];
                const double rc = a.rcut_pp ? a.rcut_pp[pl] : a.rcut;
                const double rc2 = rc * rc;
                // FP32 decisions: inside below tin, outside above tout
                tin = (float)(rc2 - a.band);
                tout = (float)(rc2 + a.band);
            }
            make_stencil<DIM>(a, x, S);
        }
        const int nb = (int)min((int64_t)32, a.n_dom - pb);
        for (int i = 0; i < nb; ++i) {
            const int64_t p = pb + i;
            const float ptin = __shfl_sync(full, tin, i), ptout = __shfl_sync(full, tout, i);
            const unsigned valid = __shfl_sync(full, S.valid, i), fastm = __shfl_sync(full, S.fast, i);
            int pc[3];
            float prc[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                pc[d] = __shfl_sync(full, S.c[d], i);
                prc[d] = __shfl_sync(full, S.rpc[d], i);
            }
            int64_t base = FILL ? rowptr[p] : 0;
            const int64_t cap = FILL ? rowptr[p + 1] - base : 0;  // the count pass's result
            int k = 0;
#pragma unroll 1
            for (int a2 = 0; a2 < 3; ++a2) {
                if (!((valid >> (6 + a2)) & 1u)) continue;
#pragma unroll 1
                for (int a1 = 0; a1 < 3; ++a1) {
                    if (!((valid >> (3 + a1)) & 1u)) continue;
#pragma unroll 1
                    for (int a0 = 0; a0 < 3; ++a0) {
                        if (!((valid >> a0) & 1u)) continue;
                        const int cc = slot_cell(pc[0], a0, a.cells.nc[0], a.geom.per[0]) +
                                       a.cells.nc[0] * (slot_cell(pc[1], a1, a.cells.nc[1], a.geom.per[1]) +
                                                        a.cells.nc[1] * slot_cell(pc[2], a2, a.cells.nc[2],
                                                                                  a.geom.per[2]));
                        const bool fast = ((fastm >> a0) & 1u) && ((fastm >> (3 + a1)) & 1u) &&
                                          ((fastm >> (6 + a2)) & 1u);
                        // x_p - corner of this cell, per axis
                        const float r0 = prc[0] - (float)(a0 - 1) * a.csf[0];
                        const float r1 = prc[1] - (float)(a1 - 1) * a.csf[1];
                        const float r2 = prc[2] - (float)(a2 - 1) * a.csf[2];
                        const int64_t cb = a.cstart[cc], ce = a.cstart[cc + 1];
                        for (int64_t t0 = cb; t0 < ce; t0 += 32) {
                            const int64_t t = t0 + lane;
                            bool acc = false, exact = false;
                            int32_t q = -1;
                            if (t < ce) {
                                q = a.cidx[t];
                                const float4 rq = a.srel[t];
                                const float o0 = r0 - rq.x;
                                float d2 = o0 * o0;
                                if (DIM > 1) {
                                    const float o1 = r1 - rq.y;
                                    d2 = fmaf(o1, o1, d2);
                                }
                                if (DIM > 2) {
                                    const float o2 = r2 - rq.z;
                                    d2 = fmaf(o2, o2, d2);
                                }
                                acc = fast && d2 < ptin;
                                exact = !acc && !(fast && d2 > ptout);  // the band, NaN, or no FP32 decision
                            }
                            // a warp-uniform branch: the FP64 test issues only
                            // when some lane needs it
                            if (__any_sync(full, exact) && exact) {
                                double o[DIM];
#pragma unroll
                                for (int d = 0; d < DIM; ++d)
                                    o[d] = offset1(a.geom, d, a.pd[p * DIM + d], a.spos[t * DIM + d]);
                                const double rc = a.rcut_pp ? a.rcut_pp[p] : a.rcut;
                                acc = norm2<DIM>(o) < rc * rc;
                            }
                            if (a.self_skip && (int64_t)q == p) acc = false;
                            const unsigned bal = __ballot_sync(full, acc);
                            if (FILL && acc) {
                                const int64_t slot = k + __popc(bal & lt_mask);
                                if (slot < cap) tmp[base + slot] = q;
                            }
                            k += __popc(bal);
                        }
                    }
                }
            }
            if (!FILL && lane == 0) {
                counts[p] = k;
                atomicMax(maxk, k);
            }
        }
    }
}

// ------------------------------------------------------------------------
// Packed variant, cells of side >= rc / 2 and a stencil of +-2 cells per
// axis (43 % fewer candidates than 3^d cells of side rc).  The cells of a
// stencil row along axis 0 are adjacent in the cell order, so each row is
// one contiguous range of the cell-ordered support; the warp concatenates
// the ranges of all rows (lane r owns row r, a warp scan gives the offsets)
// and walks the concatenation 32 candidates at a time, every lane finding
// its row by a binary search over the row ends.  Used when every periodic
// axis has at least five cells; a particle whose row would wrap around a
// periodic axis 0 walks its cells one by one.
constexpr int kPackR = 2;
constexpr int kPackW = 2 * kPackR + 1;

struct PackStencil {
    int c[3];
    float rpc[3];
    unsigned valid;  // bit kPackW d + t: slot t (offset t - kPackR) of axis d is a cell
    unsigned fast;   // bit kPackW d + t: |x_p - corner| <= 3 cell sides
    bool xwrap;      // the row along axis 0 wraps around a periodic boundary
};

template <int DIM>
__device__ __forceinline__ void make_pack_stencil(const NbrArgs& a, const double* xp, PackStencil& S) {
    S.valid = 0;
    S.fast = 0;
    S.xwrap = false;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        S.c[d] = 0;
        S.rpc[d] = 0.f;
        if (d >= DIM) {
            S.valid |= 1u << (kPackW * d + kPackR);
            S.fast |= 1u << (kPackW * d + kPackR);
            continue;
        }
        const int nc = a.cells.nc[d];
        const int c = cell_coord(xp[d], a.cells.lo[d], a.cells.cs[d], nc);
        S.c[d] = c;
        S.rpc[d] = (float)(xp[d] - (a.cells.lo[d] + (double)c * a.cells.cs[d]));
        if (d == 0 && a.geom.per[0] && (c - kPackR < 0 || c + kPackR >= nc)) S.xwrap = true;
#pragma unroll
        for (int t = 0; t < kPackW; ++t) {
            const int u = c + t - kPackR;
            const bool ok = a.geom.per[d] || (u >= 0 && u < nc);
            const double rp = xp[d] - (a.cells.lo[d] + (double)u * a.cells.cs[d]);
            if (ok) S.valid |= 1u << (kPackW * d + t);
            if (ok && a.fast && fabs(rp) <= 3.0 * a.cells.cs[d]) S.fast |= 1u << (kPackW * d + t);
        }
    }
}

__device__ __forceinline__ int pack_cell(int c, int t, int nc, int per) {
    int v = c + t - kPackR;
    if (per) v = v < 0 ? v + nc : (v >= nc ? v - nc : v);
    return v;
}

template <int DIM, bool FILL>
__global__ void __launch_bounds__(256) nbr_packed_kernel(NbrArgs a, int32_t* __restrict__ counts, int* maxk,
                                                         const int64_t* __restrict__ rowptr,
                                                         int32_t* __restrict__ tmp) {
    const int lane = threadIdx.x & 31;
    const int64_t warp0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const unsigned lt_mask = (1u << lane) - 1u;
    const unsigned full = 0xffffffffu;
    constexpr int NR = DIM == 3 ? kPackW * kPackW : (DIM == 2 ? kPackW : 1);  // stencil rows
    for (int64_t pb = warp0 * 32; pb < a.n_dom; pb += nwarps * 32) {
        float tin = 0.f, tout = 0.f;
        PackStencil S;
        {
            double x[3] = {0.0, 0.0, 0.0};
            const int64_t pl = pb + lane;
            if (pl < a.n_dom) {
#pragma unroll
                for (int d = 0; d < DIM; ++d) x[d] = a.pd[pl * DIM + d];
                const double rc = a.rcut_pp ? a.rcut_pp[pl] : a.rcut;
                const double rc2 = rc * rc;
                tin = (float)(rc2 - a.band);
                tout = (float)(rc2 + a.band);
            }
            make_pack_stencil<DIM>(a, x, S);
        }
        const int nb = (int)min((int64_t)32, a.n_dom - pb);
        for (int i = 0; i < nb; ++i) {
            const int64_t p = pb + i;
            const float ptin = __shfl_sync(full, tin, i), ptout = __shfl_sync(full, tout, i);
            const unsigned valid = __shfl_sync(full, S.valid, i), fastm = __shfl_sync(full, S.fast, i);
            const bool xwrap = __shfl_sync(full, (int)S.xwrap, i) != 0;
            int pc[3];
            float prc[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                pc[d] = __shfl_sync(full, S.c[d], i);
                prc[d] = __shfl_sync(full, S.rpc[d], i);
            }
            const int64_t base = FILL ? rowptr[p] : 0;
            const int64_t cap = FILL ? rowptr[p + 1] - base : 0;  // the count pass's result
            int k = 0;
            // classifies candidate t (valid when has) of the cell-ordered
            // support; r0..r2 = x_p - corner of its cell, fast = FP32 allowed
            auto visit = [&](bool has, int64_t t, float r0, float r1, float r2, bool fast) {
                bool acc = false, exact = false;
                int32_t q = -1;
                if (has) {
                    q = a.cidx[t];
                    const float4 rq = a.srel[t];
                    const float o0 = r0 - rq.x;
                    float d2 = o0 * o0;
                    if (DIM > 1) {
                        const float o1 = r1 - rq.y;
                        d2 = fmaf(o1, o1, d2);
                    }
                    if (DIM > 2) {
                        const float o2 = r2 - rq.z;
                        d2 = fmaf(o2, o2, d2);
                    }
                    acc = fast && d2 < ptin;
                    exact = !acc && !(fast && d2 > ptout);  // the band, NaN, or no FP32 decision
                }
                if (__any_sync(full, exact) && exact) {
                    double o[DIM];
#pragma unroll
                    for (int d = 0; d < DIM; ++d) o[d] = offset1(a.geom, d, a.pd[p * DIM + d], a.spos[t * DIM + d]);
                    const double rc = a.rcut_pp ? a.rcut_pp[p] : a.rcut;
                    acc = norm2<DIM>(o) < rc * rc;
                }
                if (a.self_skip && (int64_t)q == p) acc = false;
                const unsigned bal = __ballot_sync(full, acc);
                if (FILL && acc) {
                    const int64_t slot = k + __popc(bal & lt_mask);
                    if (slot < cap) tmp[base + slot] = q;
                }
                k += __popc(bal);
            };
            if (!xwrap) {
                // lane r < NR owns stencil row r: (a1, a2) = (r % W, r / W)
                int rlen = 0;
                int64_t rstart = 0;
                float ry = 0.f, rz = 0.f;
                int rfast = 0;
                if (lane < NR) {
                    const int a1 = DIM > 1 ? lane % kPackW : kPackR;
                    const int a2 = DIM > 2 ? lane / kPackW : kPackR;
                    if (((valid >> (kPackW + a1)) & 1u) && ((valid >> (2 * kPackW + a2)) & 1u)) {
                        const int nc0 = a.cells.nc[0];
                        const int x0 = a.geom.per[0] ? pc[0] - kPackR : max(pc[0] - kPackR, 0);
                        const int x1 = a.geom.per[0] ? pc[0] + kPackR : min(pc[0] + kPackR, nc0 - 1);
                        const int yz = DIM > 1 ? nc0 * (pack_cell(pc[1], a1, a.cells.nc[1], a.geom.per[1]) +
                                                        a.cells.nc[1] * (DIM > 2 ? pack_cell(pc[2], a2, a.cells.nc[2],
                                                                                             a.geom.per[2])
                                                                                   : 0))
                                               : 0;
                        rstart = a.cstart[x0 + yz];
                        rlen = (int)(a.cstart[x1 + yz + 1] - rstart);
                        ry = prc[1] - (float)(a1 - kPackR) * a.csf[1];
                        rz = prc[2] - (float)(a2 - kPackR) * a.csf[2];
                        rfast = ((fastm >> (kPackW + a1)) & 1u) && ((fastm >> (2 * kPackW + a2)) & 1u);
                    }
                }
                // inclusive scan of the row lengths
                int rend = rlen;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int v = __shfl_up_sync(full, rend, o);
                    if (lane >= o) rend += v;
                }
                const int total = __shfl_sync(full, rend, 31);
                for (int g0 = 0; g0 < total; g0 += 32) {
                    const int g = g0 + lane;
                    // first row whose end exceeds g
                    int lo = 0, hi = NR - 1;
#pragma unroll
                    for (int it = 0; it < 5; ++it) {
                        const int mid = (lo + hi) >> 1;
                        const int e = __shfl_sync(full, rend, mid);
                        if (lo < hi) {
                            if (e > g)
                                hi = mid;
                            else
                                lo = mid + 1;
                        }
                    }
                    const int e_r = __shfl_sync(full, rend, lo), l_r = __shfl_sync(full, rlen, lo);
                    const int64_t s_r = __shfl_sync(full, rstart, lo);
                    const float y_r = __shfl_sync(full, ry, lo), z_r = __shfl_sync(full, rz, lo);
                    const int f_r = __shfl_sync(full, rfast, lo);
                    const bool has = g < total;
                    const int64_t t = s_r + (g - (e_r - l_r));
                    // the candidate's cell along axis 0 is in its srel.w
                    int dx = 0;
                    if (has) dx = __float_as_int(a.srel[t].w) - pc[0];
                    if (a.geom.per[0]) dx = dx < -kPackR ? dx + a.cells.nc[0] : (dx > kPackR ? dx - a.cells.nc[0] : dx);
                    const bool fx = dx >= -kPackR && dx <= kPackR && ((fastm >> (dx + kPackR)) & 1u);
                    visit(has, t, prc[0] - (float)dx * a.csf[0], y_r, z_r, f_r && fx);
                }
            } else {
                // the row along the periodic axis 0 wraps: cell by cell
#pragma unroll 1
                for (int a2 = 0; a2 < kPackW; ++a2) {
                    if (!((valid >> (2 * kPackW + a2)) & 1u)) continue;
#pragma unroll 1
                    for (int a1 = 0; a1 < kPackW; ++a1) {
                        if (!((valid >> (kPackW + a1)) & 1u)) continue;
#pragma unroll 1
                        for (int a0 = 0; a0 < kPackW; ++a0) {
                            if (!((valid >> a0) & 1u)) continue;
                            const int cc = pack_cell(pc[0], a0, a.cells.nc[0], a.geom.per[0]) +
                                           a.cells.nc[0] * (pack_cell(pc[1], a1, a.cells.nc[1], a.geom.per[1]) +
                                                            a.cells.nc[1] * pack_cell(pc[2], a2, a.cells.nc[2],
                                                                                      a.geom.per[2]));
                            const bool fast = ((fastm >> a0) & 1u) && ((fastm >> (kPackW + a1)) & 1u) &&
                                              ((fastm >> (2 * kPackW + a2)) & 1u);
                            const float r0 = prc[0] - (float)(a0 - kPackR) * a.csf[0];
                            const float r1 = prc[1] - (float)(a1 - kPackR) * a.csf[1];
                            const float r2 = prc[2] - (float)(a2 - kPackR) * a.csf[2];
                            const int64_t cb = a.cstart[cc], ce = a.cstart[cc + 1];
                            for (int64_t t0 = cb; t0 < ce; t0 += 32) visit(t0 + lane < ce, t0 + lane, r0, r1, r2, fast);
                        }
                    }
                }
            }
            if (!FILL && lane == 0) {
                counts[p] = k;
                atomicMax(maxk, k);
            }
        }
    }
}

// Warp per row: rank of each entry among the row's entries -> sorted output.
__global__ void __launch_bounds__(256) sort_rows_kernel(int64_t n, const int64_t* __restrict__ rowptr,
                                                        const int32_t* __restrict__ tmp, int32_t* __restrict__ cols) {
    const int lane = threadIdx.x & 31;
    const int64_t warp0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t p = warp0; p < n; p += nwarps) {
        int64_t b = rowptr[p], e = rowptr[p + 1];
        int k = (int)(e - b);
        for (int i0 = 0; i0 < k; i0 += 32) {
            int i = i0 + lane;
            int32_t v = (i < k) ? tmp[b + i] : 0;
            int rank = 0;
            for (int j = 0; j < k; ++j) rank += (tmp[b + j] < v);
            if (i < k) cols[b + rank] = v;
        }
    }
}

// Warp per row, rows of up to 32 KPL entries: a bitonic sort in registers
// (lane l holds entries l KPL .. l KPL + KPL - 1; partners KPL or more apart
// are exchanged by shuffles).  Longer rows take the rank sort above.
template <int KPL>
__global__ void __launch_bounds__(256) sort_rows_bitonic_kernel(int64_t n, const int64_t* __restrict__ rowptr,
                                                                const int32_t* __restrict__ tmp,
                                                                int32_t* __restrict__ cols) {
    constexpr int N = 32 * KPL;
    const int lane = threadIdx.x & 31;
    const int64_t warp0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t p = warp0; p < n; p += nwarps) {
        const int64_t b = rowptr[p];
        const int k = (int)(rowptr[p + 1] - b);
        if (k > N) {
            for (int i0 = 0; i0 < k; i0 += 32) {
                const int i = i0 + lane;
                const int32_t v = (i < k) ? tmp[b + i] : 0;
                int rank = 0;
                for (int j = 0; j < k; ++j) rank += (tmp[b + j] < v);
                if (i < k) cols[b + rank] = v;
            }
            continue;
        }
        int32_t v[KPL];
#pragma unroll
        for (int s = 0; s < KPL; ++s) {
            const int e = lane * KPL + s;
            v[s] = e < k ? tmp[b + e] : INT32_MAX;
        }
#pragma unroll
        for (int size = 2; size <= N; size <<= 1) {
#pragma unroll
            for (int stride = size >> 1; stride > 0; stride >>= 1) {
                if (stride < KPL) {
#pragma unroll
                    for (int s = 0; s < KPL; ++s) {
                        const int s2 = s ^ stride;
                        if (s2 > s) {
                            const bool asc = ((lane * KPL + s) & size) == 0;
                            const int32_t x = v[s], y = v[s2];
                            if ((x > y) == asc) {
                                v[s] = y;
                                v[s2] = x;
                            }
                        }
                    }
                } else {
                    const int ls = stride / KPL;
                    const bool lower = (lane & ls) == 0;
#pragma unroll
                    for (int s = 0; s < KPL; ++s) {
                        const int32_t o = __shfl_xor_sync(0xffffffffu, v[s], ls);
                        const bool asc = ((lane * KPL + s) & size) == 0;
                        v[s] = (lower == asc) ? min(v[s], o) : max(v[s], o);
                    }
                }
            }
        }
#pragma unroll
        for (int s = 0; s < KPL; ++s) {
            const int e = lane * KPL + s;
            if (e < k) cols[b + e] = v[s];
        }
    }
}

int grid_for(int64_t items, int per_block) {
    int64_t g = (items + per_block - 1) / per_block;
    int64_t cap = (int64_t)num_sms() * 16;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

}  // namespace

// SM count of the current device, cached per device (a process may drive
// GPUs with different SM counts).
int num_sms() {
    constexpr int kDevs = 64;
    static std::atomic<int> cache[kDevs];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) dev = 0;
    std::atomic<int>* slot = dev < kDevs ? &cache[dev] : nullptr;
    int sms = slot ? slot->load(std::memory_order_relaxed) : 0;
    if (sms > 0) return sms;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) {
        cudaGetLastError();
        sms = 1;
    } else if (slot) {
        slot->store(sms, std::memory_order_relaxed);
    }
    return sms;
}

int64_t scan_tmp_elems(int64_t n) { return (n + kScanTile - 1) / kScanTile + 1; }

cudaError_t exclusive_scan_i32(const int32_t* in, int64_t n, int64_t* out, int64_t* tmp, cudaStream_t s) {
    int64_t ntiles = (n + kScanTile - 1) / kScanTile;
    if (ntiles == 0) {
        return cudaMemsetAsync(out, 0, sizeof(int64_t), s);
    }
    scan_tile_sums<<<(unsigned)ntiles, kScanThreads, 0, s>>>(in, n, tmp);
    scan_tile_offsets<<<1, kScanThreads, 0, s>>>(tmp, ntiles);
    scan_tiles<<<(unsigned)ntiles, kScanThreads, 0, s>>>(in, n, tmp, out);
    return cudaGetLastError();
}

cudaError_t bounding_box(int dim, const double* a, int64_t na, const double* b, int64_t nb, double* lo, double* hi,
                         unsigned long long* d_tmp, cudaStream_t s) {
    unsigned long long init[2 * kMaxDim];
    for (int d = 0; d < kMaxDim; ++d) {
        init[d] = ~0ull;
        init[kMaxDim + d] = 0ull;
    }
    cudaError_t e = cudaMemcpyAsync(d_tmp, init, sizeof init, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return e;
    if (na > 0) bbox_kernel<<<grid_for(na, 256), 256, 0, s>>>(dim, a, na, d_tmp);
    if (nb > 0 && b != a) bbox_kernel<<<grid_for(nb, 256), 256, 0, s>>>(dim, b, nb, d_tmp);
    unsigned long long res[2 * kMaxDim];
    e = cudaMemcpyAsync(res, d_tmp, sizeof res, cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) return e;
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return e;
    for (int d = 0; d < dim; ++d) {
        lo[d] = from_ord(res[d]);
        hi[d] = from_ord(res[kMaxDim + d]);
    }
    return cudaGetLastError();
}

cudaError_t build_cells(int dim, const double* pos, int64_t n, const CellGrid& g, int32_t* d_cell, int32_t* d_ccount,
                        int64_t* d_cstart, int64_t* d_fill, int32_t* d_cidx, double* d_spos, float4* d_srel,
                        int64_t* d_scan_tmp, cudaStream_t s) {
    int64_t ncell = (int64_t)g.nc[0] * g.nc[1] * g.nc[2];
    cudaError_t e = cudaMemsetAsync(d_ccount, 0, sizeof(int32_t) * ncell, s);
    if (e != cudaSuccess) return e;
    if (n > 0) cell_id_kernel<<<grid_for(n, 256), 256, 0, s>>>(dim, pos, n, g, d_cell, d_ccount);
    e = exclusive_scan_i32(d_ccount, ncell, d_cstart, d_scan_tmp, s);
    if (e != cudaSuccess) return e;
    e = cudaMemcpyAsync(d_fill, d_cstart, sizeof(int64_t) * ncell, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return e;
    if (n > 0)
        cell_fill_kernel<<<grid_for(n, 256), 256, 0, s>>>(dim, pos, n, d_cell, g, d_fill, d_cidx, d_spos, d_srel);
    return cudaGetLastError();
}

// Renumbering keys.  Z-order (Morton) of a particle's cell: the bits of the
// cell coordinates, shifted right by `shift`, interleaved (axis 0 lowest).
// Row-major: the index of its cell in a grid whose side is the particles'
// mean spacing, axis 0 fastest (on a jittered lattice close to the lattice's
// own order, whose consecutive rows share their neighbour offsets).
struct OrderGrid {
    int mode;                 // 0 Z-order of the list's cells, 1 row-major at the mean spacing
    int bits, shift;          // Z-order
    double lo[kMaxDim], cs[kMaxDim];
    int nc[kMaxDim];          // row-major grid
};

__device__ __forceinline__ int32_t order_key(const double* x, int dim, const CellGrid& g, const OrderGrid& o) {
    int32_t k = 0;
    if (o.mode == 0) {
        int c[kMaxDim] = {0, 0, 0};
        for (int d = 0; d < dim; ++d) c[d] = cell_coord(x[d], g.lo[d], g.cs[d], g.nc[d]);
        for (int b = 0; b < o.bits; ++b)
            for (int d = 0; d < dim; ++d) k |= ((c[d] >> (o.shift + b)) & 1) << (b * dim + d);
    } else {
        for (int d = dim - 1; d >= 0; --d) k = k * o.nc[d] + cell_coord(x[d], o.lo[d], o.cs[d], o.nc[d]);
    }
    return k;
}

__global__ void order_key_kernel(int dim, const double* __restrict__ pos, int64_t n, CellGrid g, OrderGrid o,
                                 int32_t* __restrict__ key, int32_t* __restrict__ hist) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double x[kMaxDim] = {0.0, 0.0, 0.0};
        for (int d = 0; d < dim; ++d) x[d] = pos[i * dim + d];
        const int32_t k = order_key(x, dim, g, o);
        key[i] = k;
        atomicAdd(&hist[k], 1);
    }
}

__global__ void order_scatter_kernel(const int32_t* __restrict__ key, int64_t n, int64_t* fill,
                                     int32_t* __restrict__ order) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        order[atomicAdd((unsigned long long*)&fill[key[i]], 1ull)] = (int32_t)i;
}

// the key grid of a renumbering order, and its number of keys
OrderGrid order_grid(int dim, int64_t n, const CellGrid& g, int mode, int64_t* nkeys) {
    OrderGrid o{};
    o.mode = mode;
    if (mode == 0) {
        int bits = 0;
        for (int d = 0; d < dim; ++d)
            while ((1 << bits) < g.nc[d]) ++bits;
        const int cap = kOrderKeyBits / std::max(dim, 1);
        o.shift = bits > cap ? bits - cap : 0;
        o.bits = std::min(bits, cap);
        *nkeys = (int64_t)1 << (dim * o.bits);
        return o;
    }
    double vol = 1.0;
    for (int d = 0; d < dim; ++d) vol *= g.nc[d] * g.cs[d];
    double side = std::pow(vol / (double)std::max<int64_t>(n, 1), 1.0 / dim);
    for (;;) {
        int64_t total = 1;
        for (int d = 0; d < dim; ++d) {
            o.lo[d] = g.lo[d];
            o.nc[d] = std::max(1, (int)std::ceil(g.nc[d] * g.cs[d] / side));
            o.cs[d] = g.nc[d] * g.cs[d] / o.nc[d];
            total *= o.nc[d];
        }
        if (total <= ((int64_t)1 << kOrderKeyBits)) {
            *nkeys = total;
            return o;
        }
        side *= 1.25;
    }
}

int64_t order_tmp_elems(int dim, int64_t n, const CellGrid& g, int mode) {
    int64_t nkeys = 0;
    order_grid(dim, n, g, mode, &nkeys);
    return 3 * nkeys + scan_tmp_elems(nkeys) + 1;
}

cudaError_t particle_order(int dim, const double* pos, int64_t n, const CellGrid& g, int mode, int32_t* key,
                           int64_t* tmp, int32_t* order, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    int64_t nkeys = 0;
    const OrderGrid o = order_grid(dim, n, g, mode, &nkeys);
    int32_t* hist = reinterpret_cast<int32_t*>(tmp);  // nkeys int32 in the first nkeys int64
    int64_t* starts = tmp + nkeys;                     // nkeys + 1
    int64_t* scan_tmp = starts + nkeys + 1;
    cudaError_t e = cudaMemsetAsync(hist, 0, sizeof(int32_t) * nkeys, s);
    if (e != cudaSuccess) return e;
    order_key_kernel<<<grid_for(n, 256), 256, 0, s>>>(dim, pos, n, g, o, key, hist);
    e = exclusive_scan_i32(hist, nkeys, starts, scan_tmp, s);
    if (e != cudaSuccess) return e;
    order_scatter_kernel<<<grid_for(n, 256), 256, 0, s>>>(key, n, starts, order);
    return cudaGetLastError();
}

cudaError_t count_neighbors(const NbrArgs& a, int32_t* counts, int* d_maxk, cudaStream_t s) {
    if (a.n_dom == 0) return cudaSuccess;
    int grid = grid_for(a.n_dom * 32, 256);
    if (a.packed) {
        if (a.dim == 1) nbr_packed_kernel<1, false><<<grid, 256, 0, s>>>(a, counts, d_maxk, nullptr, nullptr);
        else if (a.dim == 2) nbr_packed_kernel<2, false><<<grid, 256, 0, s>>>(a, counts, d_maxk, nullptr, nullptr);
        else nbr_packed_kernel<3, false><<<grid, 256, 0, s>>>(a, counts, d_maxk, nullptr, nullptr);
        return cudaGetLastError();
    }
    if (a.dim == 1) nbr_kernel<1, false><<<grid, 256, 0, s>>>(a, counts, d_maxk, nullptr, nullptr);
    else if (a.dim == 2) nbr_kernel<2, false><<<grid, 256, 0, s>>>(a, counts, d_maxk, nullptr, nullptr);
    else nbr_kernel<3, false><<<grid, 256, 0, s>>>(a, counts, d_maxk, nullptr, nullptr);
    return cudaGetLastError();
}

cudaError_t fill_neighbors(const NbrArgs& a, const int64_t* rowptr, int32_t* tmp, int32_t* cols, int maxk,
                           cudaStream_t s) {
    if (a.n_dom == 0) return cudaSuccess;
    int grid = grid_for(a.n_dom * 32, 256);
    if (a.packed) {
        if (a.dim == 1) nbr_packed_kernel<1, true><<<grid, 256, 0, s>>>(a, nullptr, nullptr, rowptr, tmp);
        else if (a.dim == 2) nbr_packed_kernel<2, true><<<grid, 256, 0, s>>>(a, nullptr, nullptr, rowptr, tmp);
        else nbr_packed_kernel<3, true><<<grid, 256, 0, s>>>(a, nullptr, nullptr, rowptr, tmp);
    } else if (a.dim == 1) {
        nbr_kernel<1, true><<<grid, 256, 0, s>>>(a, nullptr, nullptr, rowptr, tmp);
    } else if (a.dim == 2) {
        nbr_kernel<2, true><<<grid, 256, 0, s>>>(a, nullptr, nullptr, rowptr, tmp);
    } else {
        nbr_kernel<3, true><<<grid, 256, 0, s>>>(a, nullptr, nullptr, rowptr, tmp);
    }
    if (maxk <= 128)
        sort_rows_bitonic_kernel<4><<<grid, 256, 0, s>>>(a.n_dom, rowptr, tmp, cols);
    else if (maxk <= 256)
        sort_rows_bitonic_kernel<8><<<grid, 256, 0, s>>>(a.n_dom, rowptr, tmp, cols);
    else
        sort_rows_kernel<<<grid, 256, 0, s>>>(a.n_dom, rowptr, tmp, cols);
    return cudaGetLastError();
}

}  // namespace dcpse
