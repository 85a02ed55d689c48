// dcpse_assemble.cu -- DC-PSE kernel assembly on the device (FP64).
//
// Replaces Dcpse::initializeStaticSize (src/DCPSE/Dcpse.hpp:690-796) and the
// reference GPU path Dcpse_gpu::assembleLocalMatrices (src/DCPSE/Dcpse.cuh:
// 620-717: per-thread global scratch B, cuBLAS batched LU without pivoting,
// a separate calcKernels_gpu pass and host round trips).
//
// Particles are assembled in batches, each by three kernels that hand their
// results over through a plan-owned scratch buffer:
//  1. gram_kernel (one warp per particle)
//       eps  = (sum_q sum_d |x_pq,d|) / k / HOverEpsilon   (Vandermonde.hpp:63-81)
//       Gram A_ij = sum_q B_qi B_qj,  B_qj = E_q V_qj,
//            V_qj = m_j(x_pq/eps), E_q = exp(-|x_pq|^2 / (2 eps^2))
//            (Vandermonde.hpp:36-49, DcpseDiagonalScalingMatrix.hpp:21-41,
//             Dcpse.hpp:755-757).  Computed once over the union of the bases
//            of all terms (Dx,Dy,Dz share one basis, Dxx,Dyy,Dzz another);
//            each lane owns Gram entries and accumulates them over q in
//            neighbour order.  Written to scratch with a status word per
//            particle (4 bits per basis group).
//  2. qr_kernel (a group of LPP lanes per particle, 32/LPP particles per
//       warp): solve A a = b for every right-hand side of each basis with
//       column-pivoting Householder QR (Businger-Golub; the role of Eigen's
//       colPivHouseholderQr at Dcpse.hpp:766), columns split over the lanes
//       of the group.  The QR is a long chain of scalar steps (pivot search,
//       square root, divisions); with few lanes per particle one warp
//       instruction advances many particles, which is what the FP64 pipe of
//       this part needs.  Coefficients go back to scratch.
//  3. weights_kernel (one warp per particle)
//       K_q = exp(-|x_pq/eps|^2) sum_i a_i V_qi        (Dcpse.hpp:768-809)
//
// Every floating-point operation follows the order of the CPU oracle, and
// this translation unit is compiled with -fmad=false (fused multiply-adds are
// explicit fma calls), so the FP64 kernels equal the oracle's bit for bit
// whatever the batch size, lane grouping or CTA size.  Neighbour rows are
// processed in chunks of 32 (one row per lane), so any neighbour count is
// handled with fixed shared memory.
#include <algorithm>
#include <cstdio>

#include <cuda_bf16.h>

#include "dcpse_internal.h"

namespace dcpse {
namespace {

constexpr int kWarps = 4;  // warps per CTA of the Gram and weight kernels
constexpr int kCh = 32;    // neighbour rows per chunk
constexpr int kQrWarps = 2;  // warps per CTA of the QR kernel

// Scratch layout and shared-memory sizes of one assembly.
struct Split {
    int gstride;             // doubles of Gram entries per particle
    int cstride;             // doubles of coefficients per particle
    int nrhs[kMaxGroups];    // right-hand sides per group (per term or per output)
    int c_off[kMaxGroups];   // coefficient block of each group, [gn][nrhs]
    int nmax;                // largest basis
    int qwords;              // doubles of the largest [A|b] plus its solution block
    int pstride;             // doubles of QR work space per particle (set per lane grouping)
    int ldb;                 // row stride of the B chunk of the Gram kernel
    int nslots;              // monomial program slots per lane
    int nout;                // outputs of the plan
    int npairs;              // Gram entries per particle
    double* gram;            // [nb][gstride]
    double* coef;            // [nb][cstride]
    double* usc;             // [nb][dim][maxk] scaled offsets u = x_pq / eps of every row
    int64_t ustride;         // dim * maxk
    int maxk;
    int32_t* gst;            // [nb] group status words
    // tensor-core Gram (DCPSE_ASSEMBLE_TC): B of every particle of the batch
    // and the exponents of its columns' largest entries
    double* qws;             // global QR work space (one slot per lane group) or nullptr
    int* qperm;              // its column permutations
    bool tc;
    int kpad;                // row stride of bmat (maxk rounded up to 16)
    double* bmat;            // [nb][nu][kpad]
    int32_t* bexp;           // [nb][32]
};

template <int DIM>
__device__ __forceinline__ void load_offset(const AsmArgs& a, const double* xp, int64_t q, double* o) {
#pragma unroll
    for (int d = 0; d < DIM; ++d) o[d] = offset1(a.geom, d, xp[d], a.spos[q * DIM + d]);
}

__device__ __forceinline__ int group_status(int32_t word, int g) { return (word >> (4 * g)) & 15; }

// isfinite on the exponent bits (integer pipe, not the FP64 one)
__device__ __forceinline__ bool finite_bits(double x) { return (__double2hiint(x) & 0x7ff00000) != 0x7ff00000; }

// Tables every lane reads each row, staged in shared memory once per CTA.
struct ProgShared {
    unsigned char prog[kMaxSlots][2];
    unsigned char uslot[kMaxUnion];
};

__device__ __forceinline__ void stage_program(const AsmTables& T, ProgShared& P) {
    for (int e = threadIdx.x; e < T.nprog; e += blockDim.x) {
        P.prog[e][0] = T.prog[e][0];
        P.prog[e][1] = T.prog[e][1];
    }
    for (int e = threadIdx.x; e < T.nu; e += blockDim.x) P.uslot[e] = T.uslot[e];
    __syncthreads();
}

// Monomials of the union basis at u, into this lane's column of V
// ([slot][32]): m_j(u) = ((u0^e0) * u1^e1) * u2^e2 (Monomial.hpp:146-156)
// with the powers by ipow's squaring steps; the program performs exactly
// these multiplications, skipping factors equal to 1.0.
template <int DIM>
__device__ __forceinline__ void monomials(const double* u, double* V, const ProgShared& P, int nprog, int lane) {
#pragma unroll
    for (int d = 0; d < DIM; ++d) V[d * 32 + lane] = u[d];
    V[DIM * 32 + lane] = 1.0;
    for (int o = 0; o < nprog; ++o)
        V[(DIM + 1 + o) * 32 + lane] = V[P.prog[o][0] * 32 + lane] * V[P.prog[o][1] * 32 + lane];
}

// ----------------------------------------------------------------- 0. eps --
// One thread per particle: eps = (sum_q sum_d |x_pq,d|) / k / HOverEpsilon
// summed sequentially over q (Vandermonde::computeEps), and the status of
// each basis group (too few neighbours for that basis, or a bad eps).
template <int DIM>
__global__ void __launch_bounds__(256) eps_kernel(AsmArgs a, Split S, int64_t b0, int64_t b1) {
    const AsmTables& T = *a.tab;
    const int ngroups = T.ngroups;
    for (int64_t it = b0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; it < b1;
         it += (int64_t)gridDim.x * blockDim.x) {
        const int64_t p = a.order ? (int64_t)a.order[it] : it;
        const int64_t beg = a.rowptr[p];
        const int k = (int)(a.rowptr[p + 1] - beg);
        double xp[DIM];
#pragma unroll
        for (int d = 0; d < DIM; ++d) xp[d] = a.pos[p * DIM + d];
        double s = 0.0;
        for (int q = 0; q < k; ++q) {
            double o[DIM];
            load_offset<DIM>(a, xp, a.cols[beg + q], o);
            double acc = 0.0;
#pragma unroll
            for (int d = 0; d < DIM; ++d) acc = acc + fabs(o[d]);
            s = s + acc;
        }
        s = s / (double)k;
        double eps = s / a.h_over_eps;
        if (a.eps_fixed) eps = a.eps_fixed[p];
        int32_t word = 0;
        const bool eps_ok = (eps > 0.0) && isfinite(eps);
        for (int g = 0; g < ngroups; ++g) {
            const int st = (k < T.gn[g]) ? ST_TOO_FEW : (eps_ok ? ST_OK : ST_BAD_EPS);
            word |= st << (4 * g);
        }
        a.eps[p] = eps;
        for (int g = 0; g < ngroups; ++g) a.eip_group[(int64_t)g * a.n + p] = 1.0 / ipow(eps, (unsigned)T.gord[g]);
        S.gst[it - b0] = word;
    }
}

// ---------------------------------------------------------------- 1. Gram --
template <int DIM, int NPP>
__global__ void __launch_bounds__(256) gram_kernel(AsmArgs a, Split S, int64_t b0, int64_t b1) {
    extern __shared__ double smem[];
    __shared__ ProgShared P;
    const AsmTables& T = *a.tab;
    stage_program(T, P);
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    double* Bs = smem + (size_t)wib * (kCh * S.ldb + S.nslots * 32);
    double* V = Bs + kCh * S.ldb;
    const int nu = T.nu;
    const int npairs = T.npairs;
    const int ngroups = T.ngroups;
    const int nprog = T.nprog;

    // Gram entries owned by this lane
    int pi[NPP], pj[NPP];
#pragma unroll
    for (int t = 0; t < NPP; ++t) {
        int e = t * 32 + lane;
        pi[t] = (e < npairs) ? T.pi[e] : 0;
        pj[t] = (e < npairs) ? T.pj[e] : 0;
    }

    const int wpc = blockDim.x >> 5;
    const int64_t nw = (int64_t)gridDim.x * wpc;
    for (int64_t it = b0 + (int64_t)blockIdx.x * wpc + wib; it < b1; it += nw) {
        const int64_t slot = it - b0;
        const int64_t p = a.order ? (int64_t)a.order[it] : it;
        const int64_t beg = a.rowptr[p];
        const int k = (int)(a.rowptr[p + 1] - beg);
        const int32_t word = S.gst[slot];
        bool any_ok = false;
        for (int g = 0; g < ngroups; ++g) any_ok |= group_status(word, g) == ST_OK;
        if (!any_ok) continue;  // warp-uniform
        const double eps = a.eps[p];
        double xp[DIM];
#pragma unroll
        for (int d = 0; d < DIM; ++d) xp[d] = a.pos[p * DIM + d];

        // A_ij = sum_q B_qi B_qj, B_qj = E_q m_j(x_pq / eps)
        double acc[NPP];
#pragma unroll
        for (int t = 0; t < NPP; ++t) acc[t] = 0.0;
        for (int c0 = 0; c0 < k; c0 += kCh) {
            int q = c0 + lane;
            const int cnt = min(kCh, k - c0);
            if (q < k) {
                double o[DIM], u[DIM];
                load_offset<DIM>(a, xp, a.cols[beg + q], o);
#pragma unroll
                for (int d = 0; d < DIM; ++d) u[d] = o[d] / eps;
                double* Ur = S.usc + slot * S.ustride;
#pragma unroll
                for (int d = 0; d < DIM; ++d) Ur[d * S.maxk + q] = u[d];
                const double E = cw_exp(-norm2<DIM>(o) / (2.0 * eps * eps));
                monomials<DIM>(u, V, P, nprog, lane);
                for (int j = 0; j < nu; ++j) Bs[lane * S.ldb + j] = E * V[P.uslot[j] * 32 + lane];
            }
            __syncwarp();
            for (int r = 0; r < cnt; ++r) {
                const double* row = Bs + r * S.ldb;
#pragma unroll
                for (int t = 0; t < NPP; ++t)
                    if (t * 32 + lane < npairs) acc[t] = fma(row[pi[t]], row[pj[t]], acc[t]);
            }
            __syncwarp();
        }
        double* G = S.gram + slot * S.gstride;
#pragma unroll
        for (int t = 0; t < NPP; ++t)
            if (t * 32 + lane < npairs) G[t * 32 + lane] = acc[t];
    }
}

#include "dcpse_gram_tc.cuh"

// Gram kernel for bases whose entries do not fit in the lanes' registers
// (more than 40 x 32 pairs, e.g. 7260 for the 120-function basis of
// |alpha| = 6 in 3D): the same rows of B, and every entry's sum continued
// from the batch scratch chunk after chunk, in the same sequential order, so
// the entries equal the register version's (and the reference's) bit for bit.
template <int DIM>
__global__ void __launch_bounds__(256) gram_wide_kernel(AsmArgs a, Split S, int64_t b0, int64_t b1) {
    extern __shared__ double smem[];
    __shared__ ProgShared P;
    const AsmTables& T = *a.tab;
    stage_program(T, P);
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    double* Bs = smem + (size_t)wib * (kCh * S.ldb + S.nslots * 32);
    double* V = Bs + kCh * S.ldb;
    const int nu = T.nu;
    const int npairs = T.npairs;
    const int ngroups = T.ngroups;
    const int nprog = T.nprog;
    const int wpc = blockDim.x >> 5;
    const int64_t nw = (int64_t)gridDim.x * wpc;
    for (int64_t it = b0 + (int64_t)blockIdx.x * wpc + wib; it < b1; it += nw) {
        const int64_t slot = it - b0;
        const int64_t p = a.order ? (int64_t)a.order[it] : it;
        const int64_t beg = a.rowptr[p];
        const int k = (int)(a.rowptr[p + 1] - beg);
        const int32_t word = S.gst[slot];
        bool any_ok = false;
        for (int g = 0; g < ngroups; ++g) any_ok |= group_status(word, g) == ST_OK;
        if (!any_ok) continue;  // warp-uniform
        const double eps = a.eps[p];
        double xp[DIM];
#pragma unroll
        for (int d = 0; d < DIM; ++d) xp[d] = a.pos[p * DIM + d];
        double* G = S.gram + slot * S.gstride;
        for (int c0 = 0; c0 < k; c0 += kCh) {
            const int q = c0 + lane;
            const int cnt = min(kCh, k - c0);
            if (q < k) {
                double o[DIM], u[DIM];
                load_offset<DIM>(a, xp, a.cols[beg + q], o);
#pragma unroll
                for (int d = 0; d < DIM; ++d) u[d] = o[d] / eps;
                double* Ur = S.usc + slot * S.ustride;
#pragma unroll
                for (int d = 0; d < DIM; ++d) Ur[d * S.maxk + q] = u[d];
                const double E = cw_exp(-norm2<DIM>(o) / (2.0 * eps * eps));
                monomials<DIM>(u, V, P, nprog, lane);
                for (int j = 0; j < nu; ++j) Bs[lane * S.ldb + j] = E * V[P.uslot[j] * 32 + lane];
            }
            __syncwarp();
            for (int e = lane; e < npairs; e += 32) {
                const int pi = T.pi[e], pj = T.pj[e];
                double acc = c0 == 0 ? 0.0 : G[e];
                for (int r = 0; r < cnt; ++r) acc = fma(Bs[r * S.ldb + pi], Bs[r * S.ldb + pj], acc);
                G[e] = acc;
            }
            __syncwarp();
        }
    }
}

// B for the tensor-core products: the SIMT Gram kernel's rows of B (u, E,
// the monomial program, in the same operations), stored to bmat[slot][j][q]
// in FP64, and for every column the exponent E_j with |B_qj| < 2^E_j (from
// the largest exponent field of the column), to bexp[slot][j].  One warp per
// particle, many per SM: the FP64 work of this part needs the latency hiding.
template <int DIM>
__global__ void __launch_bounds__(256) gram_b_kernel(AsmArgs a, Split S, int64_t b0, int64_t b1) {
    extern __shared__ double smem[];
    __shared__ ProgShared P;
    const AsmTables& T = *a.tab;
    stage_program(T, P);
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    double* V = smem + (size_t)wib * (S.nslots * 32);
    const int nu = T.nu;
    const int ngroups = T.ngroups;
    const int nprog = T.nprog;
    const int wpc = blockDim.x >> 5;
    const int64_t nw = (int64_t)gridDim.x * wpc;
    for (int64_t it = b0 + (int64_t)blockIdx.x * wpc + wib; it < b1; it += nw) {
        const int64_t slot = it - b0;
        const int32_t word = S.gst[slot];
        bool any_ok = false;
        for (int g = 0; g < ngroups; ++g) any_ok |= group_status(word, g) == ST_OK;
        if (!any_ok) continue;  // warp-uniform
        const int64_t p = a.order ? (int64_t)a.order[it] : it;
        const int64_t beg = a.rowptr[p];
        const int k = (int)(a.rowptr[p + 1] - beg);
        const double eps = a.eps[p];
        double xp[DIM];
#pragma unroll
        for (int d = 0; d < DIM; ++d) xp[d] = a.pos[p * DIM + d];
        double* Bm = S.bmat + slot * (int64_t)nu * S.kpad;
        unsigned emax[kTcMaxNu];
#pragma unroll
        for (int j = 0; j < kTcMaxNu; ++j) emax[j] = 0;
        for (int c0 = 0; c0 < k; c0 += kCh) {
            const int q = c0 + lane;
            if (q < k) {
                double o[DIM], u[DIM];
                load_offset<DIM>(a, xp, a.cols[beg + q], o);
#pragma unroll
                for (int d = 0; d < DIM; ++d) u[d] = o[d] / eps;
                double* Ur = S.usc + slot * S.ustride;
#pragma unroll
                for (int d = 0; d < DIM; ++d) Ur[d * S.maxk + q] = u[d];
                const double E = cw_exp(-norm2<DIM>(o) / (2.0 * eps * eps));
                monomials<DIM>(u, V, P, nprog, lane);
#pragma unroll
                for (int j = 0; j < kTcMaxNu; ++j)
                    if (j < nu) {
                        const double b = E * V[P.uslot[j] * 32 + lane];
                        Bm[(int64_t)j * S.kpad + q] = b;
                        emax[j] = max(emax[j], ((unsigned)__double2hiint(b) >> 20) & 0x7ffu);
                    }
            }
            __syncwarp();
        }
        // |x| < 2^(e - 1022) for a normal x with exponent field e
        int mine = 0;
#pragma unroll
        for (int j = 0; j < kTcMaxNu; ++j) {
            const unsigned m = __reduce_max_sync(0xffffffffu, emax[j]);
            if (lane == j) mine = max((int)m, 1) - 1022;
        }
        S.bexp[slot * 32 + lane] = mine;
    }
}


// ------------------------------------------------------------------ 2. QR --
// All lanes of a warp run the same loop trip counts (the basis sizes are the
// plan's); particles differ only in their data, so every shuffle and warp
// barrier is reached by the whole warp.  A group whose factorisation breaks
// down (or that was not assembled) keeps running on its own work space and
// only its stores are suppressed.
template <int LPP>
__global__ void __launch_bounds__(kQrWarps * 32) qr_kernel(AsmArgs a, Split S, int64_t nb) {
    constexpr int PPW = 32 / LPP;
    extern __shared__ double smem[];
    const AsmTables& T = *a.tab;
    const bool fast = (a.flags & DCPSE_ASSEMBLE_FAST_FLAG) != 0;
    const int lane = threadIdx.x & 31;
    const int l = lane & (LPP - 1);
    const int sub = lane / LPP;
    const int wib = threadIdx.x >> 5;
    const int wpc = blockDim.x >> 5;
    const int pidx = wib * PPW + sub;  // particle slot of this lane group in the CTA
    // work space: shared memory, or a global slot per lane group when the
    // basis is too large for it (S.qws)
    const int64_t gslot = ((int64_t)blockIdx.x * wpc + wib) * PPW + sub;
    double* R = S.qws ? S.qws + gslot * S.pstride : smem + (size_t)pidx * S.pstride;
    int* perm = S.qws ? S.qperm + gslot * S.nmax
                      : reinterpret_cast<int*>(smem + (size_t)wpc * PPW * S.pstride) + pidx * S.nmax;
    const int ngroups = T.ngroups;

    for (int64_t w0 = ((int64_t)blockIdx.x * wpc + wib) * PPW; w0 < nb; w0 += (int64_t)gridDim.x * wpc * PPW) {
        const int64_t slot = w0 + sub;
        const bool valid = slot < nb;
        int32_t word = valid ? S.gst[slot] : 0x11111111;
        const double* G = S.gram + (valid ? slot : 0) * S.gstride;
        for (int g = 0; g < ngroups; ++g) {
            const int n = T.gn[g];
            const int nrhs = S.nrhs[g];
            const int ncol = n + nrhs;
            const int ldr = ncol;         // [A | b...], n rows
            double* Z = R + n * ncol;     // solutions, n x nrhs
            const bool active = valid && group_status(word, g) == ST_OK;
            // R = [A | b...]
            for (int e = l; e < n * ncol; e += LPP) {
                const int i = e / ncol, j = e - i * ncol;
                double v = 0.0;
                if (active) {
                    if (j < n) {
                        const int ui = T.gidx[g][i], uj = T.gidx[g][j];
                        v = G[T.upair[min(ui, uj)][max(ui, uj)]];
                    } else {
                        v = fast ? T.b_out[g][j - n][i] : T.b_term[g][j - n][i];
                    }
                }
                R[i * ldr + j] = v;
            }
            for (int i = l; i < n; i += LPP) perm[i] = i;
            __syncwarp();
            bool dead = !active;
            for (int kk = 0; kk < n; ++kk) {
                // column norms of the trailing block, pivot = first largest
                double best = -1.0;
                int bidx = 0x7fffffff;
                for (int j = kk + ((l - kk) & (LPP - 1)); j < n; j += LPP) {
                    double sn = 0.0;
                    for (int i = kk; i < n; ++i) sn = fma(R[i * ldr + j], R[i * ldr + j], sn);
                    if (sn > best) {
                        best = sn;
                        bidx = j;
                    }
                }
#pragma unroll
                for (int o = LPP / 2; o > 0; o >>= 1) {
                    double ob = __shfl_xor_sync(0xffffffffu, best, o);
                    int oi = __shfl_xor_sync(0xffffffffu, bidx, o);
                    if (ob > best || (ob == best && oi < bidx)) {
                        best = ob;
                        bidx = oi;
                    }
                }
                const int piv = (bidx == 0x7fffffff) ? kk : bidx;
                // sigma = the pivot column's norm (NaN when all norms were NaN)
                double sigma;
                if (bidx == 0x7fffffff) {
                    double sn = 0.0;
                    for (int i = kk; i < n; ++i) sn = fma(R[i * ldr + kk], R[i * ldr + kk], sn);
                    sigma = sn;
                } else {
                    sigma = best;
                }
                dead |= !(sigma > 0.0);
                if (piv != kk) {
                    for (int i = l; i < n; i += LPP) {
                        const double t0 = R[i * ldr + kk];
                        R[i * ldr + kk] = R[i * ldr + piv];
                        R[i * ldr + piv] = t0;
                    }
                    if (l == 0) {
                        const int t0 = perm[kk];
                        perm[kk] = perm[piv];
                        perm[piv] = t0;
                    }
                }
                __syncwarp();
                const double alpha = R[kk * ldr + kk];
                const double nr = sqrt(sigma);
                const double beta = (alpha >= 0.0) ? -nr : nr;
                const double den = alpha - beta;
                const double tau = (beta - alpha) / beta;
                __syncwarp();
                for (int i = kk + 1 + l; i < n; i += LPP) R[i * ldr + kk] = R[i * ldr + kk] / den;
                __syncwarp();
                if (l == 0) R[kk * ldr + kk] = beta;
                for (int j = kk + 1 + l; j < ncol; j += LPP) {
                    double sv = R[kk * ldr + j];
                    for (int i = kk + 1; i < n; ++i) sv = fma(R[i * ldr + kk], R[i * ldr + j], sv);
                    sv = sv * tau;
                    R[kk * ldr + j] = R[kk * ldr + j] - sv;
                    for (int i = kk + 1; i < n; ++i) R[i * ldr + j] = fma(-sv, R[i * ldr + kk], R[i * ldr + j]);
                }
                __syncwarp();
            }
            // back substitution, right-hand sides split over the lanes
            for (int r = l; r < nrhs; r += LPP) {
                for (int i = n - 1; i >= 0; --i) {
                    double sv = R[i * ldr + n + r];
                    for (int j = i + 1; j < n; ++j) sv = fma(-R[i * ldr + j], Z[j * nrhs + r], sv);
                    Z[i * nrhs + r] = sv / R[i * ldr + i];
                }
            }
            __syncwarp();
            if (!dead) {
                double* C = S.coef + slot * S.cstride + S.c_off[g];
                for (int e = l; e < n * nrhs; e += LPP) {
                    const int i = e / nrhs, r = e - i * nrhs;
                    C[perm[i] * nrhs + r] = Z[i * nrhs + r];
                }
            } else if (active) {
                word = (word & ~(15 << (4 * g))) | (ST_SINGULAR << (4 * g));
            }
            __syncwarp();
        }
        if (valid && l == 0) S.gst[slot] = word;
    }
}

// ------------------------------------------------------------- 3. weights --
// One warp per particle, one neighbour row per lane.  The right-hand sides
// and outputs are run-time loops (no work predicated off on the FP64 pipe);
// per-output sums live in this lane's column of shared memory.
template <int DIM>
__global__ void __launch_bounds__(256) weights_kernel(AsmArgs a, Split S, int64_t b0, int64_t b1) {
    extern __shared__ double smem[];
    __shared__ ProgShared P;
    const AsmTables& T = *a.tab;
    stage_program(T, P);
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    double* Cs = smem + (size_t)wib * (S.cstride + (S.nslots + S.nout) * 32);
    double* V = Cs + S.cstride;
    double* Wacc = V + S.nslots * 32;
    const int ngroups = T.ngroups;
    const int nprog = T.nprog;
    const bool fast = (a.flags & DCPSE_ASSEMBLE_FAST_FLAG) != 0;
    const bool st_terms = a.k_term != nullptr;
    const int noutputs = T.noutputs;

    const int wpc = blockDim.x >> 5;
    const int64_t nw = (int64_t)gridDim.x * wpc;
    for (int64_t it = b0 + (int64_t)blockIdx.x * wpc + wib; it < b1; it += nw) {
        const int64_t slot = it - b0;
        const int64_t p = a.order ? (int64_t)a.order[it] : it;
        const int64_t beg = a.rowptr[p];
        const int k = (int)(a.rowptr[p + 1] - beg);
        const double eps = a.eps[p];
        const int32_t word = S.gst[slot];
        for (int e = lane; e < S.cstride; e += 32) Cs[e] = S.coef[slot * S.cstride + e];
        __syncwarp();

        double eipg[kMaxGroups];
#pragma unroll
        for (int g = 0; g < kMaxGroups; ++g) eipg[g] = (g < ngroups) ? 1.0 / ipow(eps, (unsigned)T.gord[g]) : 0.0;
        bool nonfinite = false;
        for (int c0 = 0; c0 < k; c0 += kCh) {
            int q = c0 + lane;
            if (q >= k) break;  // rows of this lane are done; no warp sync below
            // u = x_pq / eps as the Gram kernel computed it (rows of particles
            // with no assembled group were skipped there and are not used here)
            double u[DIM];
            const double* Ur = S.usc + slot * S.ustride;
#pragma unroll
            for (int d = 0; d < DIM; ++d) u[d] = Ur[d * S.maxk + q];
            monomials<DIM>(u, V, P, nprog, lane);
            const double ef = cw_exp(-norm2<DIM>(u));
            for (int t = 0; t < noutputs; ++t) Wacc[t * 32 + lane] = 0.0;
            for (int g = 0; g < ngroups; ++g) {
                const int n = T.gn[g];
                const int nrhs = S.nrhs[g];
                const bool ok = group_status(word, g) == ST_OK;
                const double* Ag = Cs + S.c_off[g];
                double eip = eipg[0];
#pragma unroll
                for (int t = 1; t < kMaxGroups; ++t)
                    if (t == g) eip = eipg[t];
                for (int r = 0; r < nrhs; ++r) {
                    double res = 0.0;
                    if (ok) {
                        if (fast) {
                            for (int i = 0; i < n; ++i)
                                res = fma(Ag[i * nrhs + r], V[P.uslot[T.gidx[g][i]] * 32 + lane], res);
                        } else {
                            for (int i = 0; i < n; ++i) {
                                double t0 = Ag[i * nrhs + r] * V[P.uslot[T.gidx[g][i]] * 32 + lane];
                                t0 = t0 * ef;
                                res = res + t0;
                            }
                        }
                    }
                    double Kq;
                    int o2;
                    if (fast) {
                        Kq = ok ? (res * ef) : 0.0;
                        o2 = T.out_of_rhs[g][r];
                    } else {
                        Kq = res;
                        const int term = T.term_of_rhs[g][r];
                        if (st_terms) a.k_term[(int64_t)term * a.nnz + beg + q] = Kq;
                        o2 = T.term_output[term];
                    }
                    nonfinite |= !finite_bits(Kq);
                    Wacc[o2 * 32 + lane] = Wacc[o2 * 32 + lane] + Kq * eip;
                }
            }
            for (int t = 0; t < noutputs; ++t) {
                const double w = Wacc[t * 32 + lane];
                if (a.w64) a.w64[(int64_t)t * a.nnz + beg + q] = w;
                const float w32 = (float)w;
                if (a.w32) a.w32[(int64_t)t * a.nnz + beg + q] = w32;
                if (a.r16)
                    reinterpret_cast<__nv_bfloat16*>(a.r16)[(int64_t)t * a.nnz + beg + q] =
                        __float2bfloat16_rn((float)(w - (double)w32));
                if (a.r32) a.r32[(int64_t)t * a.nnz + beg + q] = (float)(w - (double)w32);
            }
        }
        nonfinite = __any_sync(0xffffffffu, nonfinite);
        if (nonfinite) {
            // zero every stored row of this particle (the oracle zeroes the
            // affected term's kernels; fused outputs are zeroed entirely)
            for (int q = lane; q < k; q += 32) {
                if (st_terms)
                    for (int t = 0; t < T.nterms; ++t) a.k_term[(int64_t)t * a.nnz + beg + q] = 0.0;
                for (int t = 0; t < noutputs; ++t) {
                    if (a.w64) a.w64[(int64_t)t * a.nnz + beg + q] = 0.0;
                    if (a.w32) a.w32[(int64_t)t * a.nnz + beg + q] = 0.0f;
                    if (a.r16)
                        reinterpret_cast<__nv_bfloat16*>(a.r16)[(int64_t)t * a.nnz + beg + q] = __float2bfloat16_rn(0.0f);
                    if (a.r32) a.r32[(int64_t)t * a.nnz + beg + q] = 0.0f;
                }
            }
        }
        if (lane == 0) {
            int st = ST_OK;
            for (int g = 0; g < ngroups; ++g)
                if (st == ST_OK && group_status(word, g) != ST_OK) st = group_status(word, g);
            if (st == ST_OK && nonfinite) st = ST_NONFINITE;
            a.status[p] = st;
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------- launches --
int warps_of(const AsmArgs& a) { return (a.warps == 2 || a.warps == 8) ? a.warps : kWarps; }

int smem_attr(cudaDeviceAttr attr, int fallback) {
    int dev = 0, v = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&v, attr, dev) != cudaSuccess) return fallback;
    return v;
}

template <typename K>
cudaError_t persistent(K kern, int threads, size_t bytes, int64_t work_per_cta, int64_t units, int& grid_out) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, bytes);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    int64_t need = (units + work_per_cta - 1) / work_per_cta;
    int64_t grid = (int64_t)num_sms() * per_sm;
    if (grid > need) grid = need;
    if (grid < 1) grid = 1;
    grid_out = (int)grid;
    return cudaSuccess;
}

template <int DIM>
cudaError_t launch_eps(const AsmArgs& a, const Split& S, int64_t b0, int64_t b1, cudaStream_t s) {
    auto kern = eps_kernel<DIM>;
    int grid = 0;
    cudaError_t e = persistent(kern, 256, 0, 256, b1 - b0, grid);
    if (e != cudaSuccess) return e;
    kern<<<grid, 256, 0, s>>>(a, S, b0, b1);
    return cudaGetLastError();
}

template <int DIM, int NPP>
cudaError_t launch_gram(const AsmArgs& a, const Split& S, int64_t b0, int64_t b1, cudaStream_t s) {
    int warps = warps_of(a);
    const size_t per_warp = (size_t)(kCh * S.ldb + S.nslots * 32) * sizeof(double);
    if constexpr (NPP == 0) {
        // large bases: as many warps as their B chunks leave room for
        const int fit = smem_attr(cudaDevAttrMaxSharedMemoryPerBlockOptin, 227 * 1024) / (int)per_warp;
        warps = std::max(1, std::min(warps, fit));
        const size_t bytes = per_warp * warps;
        auto kern = gram_wide_kernel<DIM>;
        int grid = 0;
        cudaError_t e = persistent(kern, warps * 32, bytes, warps, b1 - b0, grid);
        if (e != cudaSuccess) return e;
        kern<<<grid, warps * 32, bytes, s>>>(a, S, b0, b1);
        return cudaGetLastError();
    }
    const size_t bytes = per_warp * warps;
    auto kern = gram_kernel<DIM, NPP == 0 ? 1 : NPP>;
    int grid = 0;
    cudaError_t e = persistent(kern, warps * 32, bytes, warps, b1 - b0, grid);
    if (e != cudaSuccess) return e;
    kern<<<grid, warps * 32, bytes, s>>>(a, S, b0, b1);
    return cudaGetLastError();
}

// Work space of one particle: [A|b] then the solutions of the largest group,
// padded to LPP mod 16 doubles so that the lane groups of a half warp (16
// lanes, 64-bit accesses) fall on distinct shared-memory banks.
int qr_pstride(const Split& S, int lpp) { return S.qwords + ((lpp - S.qwords) & 15); }

size_t qr_bytes(const Split& S, int lpp) {
    return (size_t)kQrWarps * (32 / lpp) * (qr_pstride(S, lpp) * sizeof(double) + S.nmax * sizeof(int));
}

// CTAs per SM of the QR with its work space in global memory (one warp and
// one particle each)
constexpr int kQrGlobalPerSm = 4;

template <int LPP>
cudaError_t launch_qr(const AsmArgs& a, Split S, int64_t nb, cudaStream_t s) {
    constexpr int PPW = 32 / LPP;
    S.pstride = qr_pstride(S, LPP);
    if (S.qws) {
        const int64_t grid = std::min<int64_t>((int64_t)num_sms() * kQrGlobalPerSm, nb);
        qr_kernel<LPP><<<(unsigned)std::max<int64_t>(grid, 1), 32, 0, s>>>(a, S, nb);
        return cudaGetLastError();
    }
    const size_t bytes = qr_bytes(S, LPP);
    auto kern = qr_kernel<LPP>;
    int grid = 0;
    cudaError_t e = persistent(kern, kQrWarps * 32, bytes, (int64_t)kQrWarps * PPW, nb, grid);
    if (e != cudaSuccess) return e;
    kern<<<grid, kQrWarps * 32, bytes, s>>>(a, S, nb);
    return cudaGetLastError();
}

template <int DIM>
cudaError_t launch_weights(const AsmArgs& a, const Split& S, int64_t b0, int64_t b1, cudaStream_t s) {
    int warps = warps_of(a);
    const size_t per_warp = (size_t)(S.cstride + (S.nslots + S.nout) * 32) * sizeof(double);
    // large bases: as many warps as their coefficients and monomials leave room for
    warps = std::max(1, std::min(warps, smem_attr(cudaDevAttrMaxSharedMemoryPerBlockOptin, 227 * 1024) / (int)per_warp));
    const size_t bytes = per_warp * warps;
    auto kern = weights_kernel<DIM>;
    int grid = 0;
    cudaError_t e = persistent(kern, warps * 32, bytes, warps, b1 - b0, grid);
    if (e != cudaSuccess) return e;
    kern<<<grid, warps * 32, bytes, s>>>(a, S, b0, b1);
    return cudaGetLastError();
}

// lanes per particle of the QR: the fewest that still leave >= 6 warps per SM
// resident within the shared-memory budget (on the 128^3 gradient+Laplacian
// cloud 4 lanes / 6 warps beat 8 lanes / 12 warps and 2 lanes / 2 warps)
int qr_lanes_auto(const Split& S) {
    const int per_sm = smem_attr(cudaDevAttrMaxSharedMemoryPerMultiprocessor, 228 * 1024);
    const int per_block = smem_attr(cudaDevAttrMaxSharedMemoryPerBlockOptin, 227 * 1024);
    for (int lpp : {1, 2, 4, 8, 16}) {
        const size_t b = qr_bytes(S, lpp);
        if (b > (size_t)per_block) continue;
        const int blocks = (int)(per_sm / (b + 1024));
        if (blocks * kQrWarps >= 6) return lpp;
    }
    return 32;
}

cudaError_t launch_qr_any(const AsmArgs& a, const Split& S, int lpp, int64_t nb, cudaStream_t s) {
    switch (lpp) {
        case 1: return launch_qr<1>(a, S, nb, s);
        case 2: return launch_qr<2>(a, S, nb, s);
        case 4: return launch_qr<4>(a, S, nb, s);
        case 8: return launch_qr<8>(a, S, nb, s);
        case 16: return launch_qr<16>(a, S, nb, s);
        default: return launch_qr<32>(a, S, nb, s);
    }
}

template <int DIM>
cudaError_t launch_gram_tc(const AsmArgs& a, const Split& S, int64_t b0, int64_t b1, cudaStream_t s) {
    {
        const int warps = warps_of(a);
        const size_t bytes = (size_t)(S.nslots * 32) * sizeof(double) * warps;
        auto kb = gram_b_kernel<DIM>;
        int grid = 0;
        cudaError_t e = persistent(kb, warps * 32, bytes, warps, b1 - b0, grid);
        if (e != cudaSuccess) return e;
        kb<<<grid, warps * 32, bytes, s>>>(a, S, b0, b1);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    const TcLayout L = tc_layout(S.maxk, S.npairs);
    auto kern = gram_tc_kernel;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.bytes);
    if (e != cudaSuccess) return e;
    // one CTA per SM holds all its tensor memory, two particles per CTA at a time
    const int64_t grid = std::min<int64_t>((b1 - b0 + 1) / 2, (int64_t)num_sms());
    kern<<<(unsigned)grid, kTcThreads, L.bytes, s>>>(a, S, b0, b1, L);
    return cudaGetLastError();
}

template <int DIM, int NPP>
cudaError_t run(const AsmArgs& a, const AsmTables& h, const Split& S, int lpp, cudaStream_t s) {
    for (int64_t b0 = 0; b0 < a.n; b0 += a.scratch_particles) {
        const int64_t b1 = std::min(a.n, b0 + a.scratch_particles);
        cudaError_t e = launch_eps<DIM>(a, S, b0, b1, s);
        if (e == cudaSuccess)
            e = S.tc ? launch_gram_tc<DIM>(a, S, b0, b1, s) : launch_gram<DIM, NPP>(a, S, b0, b1, s);
        if (e == cudaSuccess) e = launch_qr_any(a, S, lpp, b1 - b0, s);
        if (e == cudaSuccess) e = launch_weights<DIM>(a, S, b0, b1, s);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

template <int DIM>
cudaError_t dispatch(const AsmArgs& a, const AsmTables& h, const Split& S, int lpp, cudaStream_t s) {
    // Gram entries per lane: the smallest instantiated count that holds them
    // all (a slot no lane uses would still occupy the FP64 pipe every row)
    const int npp = (h.npairs + 31) / 32;
    if (npp <= 2) return run<DIM, 2>(a, h, S, lpp, s);
    if (npp <= 4) return run<DIM, 4>(a, h, S, lpp, s);
    if (npp <= 7) return run<DIM, 7>(a, h, S, lpp, s);
    if (npp <= 8) return run<DIM, 8>(a, h, S, lpp, s);
    if (npp <= 16) return run<DIM, 16>(a, h, S, lpp, s);
    if (npp <= 40) return run<DIM, 40>(a, h, S, lpp, s);
    return run<DIM, 0>(a, h, S, lpp, s);  // the wide Gram kernel
}

Split make_split(const AsmTables& h, int flags) {
    Split S{};
    const bool fast = (flags & DCPSE_ASSEMBLE_FAST_FLAG) != 0;
    S.gstride = (h.npairs + 1) & ~1;
    S.nmax = 1;
    S.qwords = 1;
    int off = 0;
    for (int g = 0; g < h.ngroups; ++g) {
        const int n = h.gn[g];
        S.nrhs[g] = fast ? h.nout_rhs[g] : h.nterm_rhs[g];
        S.c_off[g] = off;
        off += n * S.nrhs[g];
        S.nmax = std::max(S.nmax, n);
        S.qwords = std::max(S.qwords, n * (n + S.nrhs[g]) + n * S.nrhs[g]);
    }
    S.cstride = (off + 1) & ~1;
    S.ldb = h.nu | 1;
    S.nslots = h.nslots;
    S.nout = h.noutputs;
    S.npairs = h.npairs;
    return S;
}

int tc_kpad(int maxk) { return ((std::max(maxk, 1) + 15) / 16) * 16; }

}  // namespace

bool assembly_uses_tc(const AsmTables& h, int flags, int maxk) {
    if (!(flags & DCPSE_ASSEMBLE_TC) || !(flags & DCPSE_ASSEMBLE_FAST_FLAG) || h.nu > kTcMaxNu || maxk > kTcMaxK)
        return false;
    // the planes, the monomial scratch and the pair sums fit in one CTA
    const TcLayout L = tc_layout(maxk, h.npairs);
    return L.bytes + 4096 <= (size_t)smem_attr(cudaDevAttrMaxSharedMemoryPerBlockOptin, 227 * 1024);
}

int64_t assembly_scratch_bytes(const AsmTables& h, int flags, int maxk) {
    const Split S = make_split(h, flags);
    int64_t b = (int64_t)(S.gstride + S.cstride + (int64_t)h.dim * std::max(maxk, 1)) * (int64_t)sizeof(double) +
                (int64_t)sizeof(int32_t);
    if (assembly_uses_tc(h, flags, maxk))
        b += (int64_t)h.nu * tc_kpad(maxk) * (int64_t)sizeof(double) + 32 * (int64_t)sizeof(int32_t);
    return b;
}

int64_t assembly_qr_ws_bytes(const AsmTables& h, int flags) {
    Split S = make_split(h, flags);
    if (qr_bytes(S, 32) <= (size_t)smem_attr(cudaDevAttrMaxSharedMemoryPerBlockOptin, 227 * 1024)) return 0;
    const int64_t slots = (int64_t)num_sms() * kQrGlobalPerSm;
    return slots * ((int64_t)qr_pstride(S, 32) * (int64_t)sizeof(double) + (int64_t)S.nmax * (int64_t)sizeof(int));
}

int64_t binning_tmp_elems(int64_t n, int maxk, int width) {
    const int64_t nb = maxk / (width > 0 ? width : 1) + 1;
    return nb + 1 + scan_tmp_elems(nb);
}

namespace {
__global__ void khist_kernel(const int64_t* __restrict__ rowptr, int64_t n, int width, int32_t* __restrict__ hist) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(&hist[(int)(rowptr[p + 1] - rowptr[p]) / width], 1);
}

__global__ void kscatter_kernel(const int64_t* __restrict__ rowptr, int64_t n, int width, int64_t* fill,
                                int32_t* __restrict__ order) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
        const int b = (int)(rowptr[p + 1] - rowptr[p]) / width;
        order[atomicAdd((unsigned long long*)&fill[b], 1ull)] = (int32_t)p;
    }
}
}  // namespace

cudaError_t bin_by_count(const int64_t* rowptr, int64_t n, int maxk, int width, int32_t* order, int32_t* hist,
                         int64_t* tmp64, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    if (width < 1) width = 1;
    const int64_t nb = maxk / width + 1;
    int64_t* starts = tmp64;            // nb + 1
    int64_t* scan_tmp = tmp64 + nb + 1;
    cudaError_t e = cudaMemsetAsync(hist, 0, sizeof(int32_t) * nb, s);
    if (e != cudaSuccess) return e;
    const int grid = (int)std::min<int64_t>((n + 255) / 256, (int64_t)num_sms() * 8);
    khist_kernel<<<grid, 256, 0, s>>>(rowptr, n, width, hist);
    e = exclusive_scan_i32(hist, nb, starts, scan_tmp, s);
    if (e != cudaSuccess) return e;
    kscatter_kernel<<<grid, 256, 0, s>>>(rowptr, n, width, starts, order);
    return cudaGetLastError();
}

cudaError_t assemble(const AsmArgs& a, const AsmTables& h, cudaStream_t s) {
    if (a.n == 0) return cudaSuccess;
    if (!a.scratch || a.scratch_particles < 1) return cudaErrorInvalidValue;
    Split S = make_split(h, a.flags);
    const int64_t nb = a.scratch_particles;
    S.gram = a.scratch;
    S.coef = S.gram + nb * S.gstride;
    S.maxk = std::max(a.maxk, 1);
    S.ustride = (int64_t)h.dim * S.maxk;
    S.usc = S.coef + nb * S.cstride;
    S.tc = assembly_uses_tc(h, a.flags, a.maxk);
    if (S.tc) {
        S.kpad = tc_kpad(a.maxk);
        S.bmat = S.usc + nb * S.ustride;
        S.bexp = reinterpret_cast<int32_t*>(S.bmat + nb * (int64_t)h.nu * S.kpad);
        S.gst = S.bexp + nb * 32;
    } else {
        S.gst = reinterpret_cast<int32_t*>(S.usc + nb * S.ustride);
    }
    int lpp = a.qr_lanes;
    if (lpp != 1 && lpp != 2 && lpp != 4 && lpp != 8 && lpp != 16 && lpp != 32) lpp = qr_lanes_auto(S);
    if (a.qws) {
        // large bases: one warp per particle, the work space in global memory
        lpp = 32;
        S.qws = a.qws;
        S.qperm = reinterpret_cast<int*>(a.qws + (int64_t)num_sms() * kQrGlobalPerSm * qr_pstride(S, 32));
    } else if (qr_bytes(S, lpp) > (size_t)smem_attr(cudaDevAttrMaxSharedMemoryPerBlockOptin, 227 * 1024)) {
        // a lane grouping whose work space does not fit is refused before any launch
        return cudaErrorInvalidConfiguration;
    }
    if (h.dim == 3) return dispatch<3>(a, h, S, lpp, s);
    if (h.dim == 2) return dispatch<2>(a, h, S, lpp, s);
    return dispatch<1>(a, h, S, lpp, s);
}

}  // namespace dcpse
