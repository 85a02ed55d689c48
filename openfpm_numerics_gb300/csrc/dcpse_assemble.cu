// dcpse_assemble.cu -- DC-PSE kernel assembly on the device (FP64).
//
// Replaces Dcpse::initializeStaticSize (src/DCPSE/Dcpse.hpp:690-796) and the
// reference GPU path Dcpse_gpu::assembleLocalMatrices (src/DCPSE/Dcpse.cuh:
// 620-717: per-thread global scratch B, cuBLAS batched LU without pivoting,
// a separate calcKernels_gpu pass and host round trips).
//
// One warp per particle, persistent grid.  For particle p with k neighbours:
//  1. eps   = (sum_q sum_d |x_pq,d|) / k / HOverEpsilon   (Vandermonde.hpp:63-81)
//  2. Gram  A_ij = sum_q B_qi B_qj,  B_qj = E_q V_qj,
//           V_qj = m_j(x_pq/eps), E_q = exp(-|x_pq|^2 / (2 eps^2))
//           (Vandermonde.hpp:36-49, DcpseDiagonalScalingMatrix.hpp:21-41,
//            Dcpse.hpp:755-757).  Computed once over the union of the bases
//           of all terms of the plan (Dx,Dy,Dz share one basis, Dxx,Dyy,Dzz
//           another); each lane owns Gram entries and accumulates them over q
//           in neighbour order.
//  3. Solve A a = b for every right-hand side of each basis with a
//           warp-parallel column-pivoting Householder QR (Businger-Golub; the
//           role of Eigen's colPivHouseholderQr at Dcpse.hpp:766).
//  4. K_q = exp(-|x_pq/eps|^2) sum_i a_i V_qi        (Dcpse.hpp:768-809)
//
// Every floating-point operation follows the order of the CPU oracle, and
// this translation unit is compiled with -fmad=false (fused multiply-adds are
// explicit fma calls), so the FP64 kernels equal the oracle's bit for bit.
// Neighbour rows are processed in chunks of 32 (one row per lane), so any
// neighbour count is handled with fixed shared memory.
#include <algorithm>
#include <cstdio>

#include <cuda_bf16.h>

#include "dcpse_internal.h"

namespace dcpse {
namespace {

constexpr int kWarps = 4;  // warps per CTA
constexpr int kCh = 32;    // neighbour rows per chunk
constexpr int kRhs = 8;    // right-hand sides per basis held in registers

struct Layout {
    int ldb;        // row stride of the B chunk (doubles)
    int ldr;        // row stride of the QR work matrix
    int nmax;       // largest basis
    int off_b, off_g, off_r, off_z, off_a, off_perm, words;  // offsets in doubles
    int a_off[kMaxGroups];  // coefficient block of each group inside A region
};

__device__ __forceinline__ double sel_pow(const double (&pw)[8], int e, int maxe) {
    double r = pw[0];
#pragma unroll
    for (int t = 1; t < 8; ++t)
        if (t < maxe) r = (e == t) ? pw[t] : r;
    return r;
}

template <int DIM, int MAXE>
__device__ __forceinline__ void powers(const double* u, double (&pw)[kMaxDim][8]) {
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
#pragma unroll
        for (int e = 0; e < 8; ++e) pw[d][e] = (e < MAXE) ? ipow(u[d], (unsigned)e) : 0.0;
    }
}

// m_j(u) = ((scalar * u0^e0) * u1^e1) * u2^e2 with scalar 1 (Monomial.hpp:146-156)
template <int DIM, int MAXE>
__device__ __forceinline__ double mono(const double (&pw)[kMaxDim][8], const unsigned char* e) {
    double r = 1.0;
#pragma unroll
    for (int d = 0; d < DIM; ++d) r = r * sel_pow(pw[d], e[d], MAXE);
    return r;
}

template <int DIM>
__device__ __forceinline__ void load_offset(const AsmArgs& a, const double* xp, int64_t q, double* o) {
#pragma unroll
    for (int d = 0; d < DIM; ++d) o[d] = offset1(a.geom, d, xp[d], a.pos[q * DIM + d]);
}

template <int DIM, int MAXE, int NPP>
__global__ void __launch_bounds__(256) assemble_kernel(AsmArgs a, Layout L) {
    extern __shared__ double smem[];
    const AsmTables& T = *a.tab;
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    double* S = smem + (size_t)wib * L.words;
    double* Bs = S + L.off_b;
    double* Gs = S + L.off_g;
    double* R = S + L.off_r;
    double* Z = S + L.off_z;
    double* Acoef = S + L.off_a;
    int* perm = reinterpret_cast<int*>(S + L.off_perm);

    const int nu = T.nu;
    const int npairs = T.npairs;
    const int ngroups = T.ngroups;
    const bool fast = (a.flags & DCPSE_ASSEMBLE_FAST_FLAG) != 0;
    const bool st_terms = a.k_term != nullptr;
    const int noutputs = T.noutputs;

    // Gram entries owned by this lane
    int pi[NPP], pj[NPP];
#pragma unroll
    for (int t = 0; t < NPP; ++t) {
        int e = t * 32 + lane;
        pi[t] = (e < npairs) ? T.pi[e] : 0;
        pj[t] = (e < npairs) ? T.pj[e] : 0;
    }

    const int wpc = blockDim.x >> 5;
    const int64_t gw = ((int64_t)blockIdx.x * wpc + wib);
    const int64_t nw = (int64_t)gridDim.x * wpc;
    for (int64_t it = gw; it < a.n; it += nw) {
        const int64_t p = a.order ? (int64_t)a.order[it] : it;
        const int64_t beg = a.rowptr[p];
        const int k = (int)(a.rowptr[p + 1] - beg);
        double xp[DIM];
#pragma unroll
        for (int d = 0; d < DIM; ++d) xp[d] = a.pos[p * DIM + d];

        // ---- 1. eps (sequential sum over q, as Vandermonde::computeEps) ----
        double s = 0.0;
        for (int c0 = 0; c0 < k; c0 += kCh) {
            int q = c0 + lane;
            double v = 0.0;
            if (q < k) {
                double o[DIM];
                load_offset<DIM>(a, xp, a.cols[beg + q], o);
                double acc = 0.0;
#pragma unroll
                for (int d = 0; d < DIM; ++d) acc = acc + fabs(o[d]);
                v = acc;
            }
            int cnt = min(kCh, k - c0);
            for (int t = 0; t < kCh; ++t) {
                double w = __shfl_sync(0xffffffffu, v, t);
                if (t < cnt) s = s + w;
            }
        }
        s = s / (double)k;
        double eps = s / a.h_over_eps;
        if (a.eps_fixed) eps = a.eps_fixed[p];
        // per-group status: too few neighbours for that basis, or bad eps
        int gst[kMaxGroups];
        bool any_ok = false;
        const bool eps_ok = (eps > 0.0) && isfinite(eps);
        for (int g = 0; g < ngroups; ++g) {
            gst[g] = (k < T.gn[g]) ? ST_TOO_FEW : (eps_ok ? ST_OK : ST_BAD_EPS);
            any_ok |= (gst[g] == ST_OK);
        }
        if (lane == 0) {
            a.eps[p] = eps;
            for (int g = 0; g < ngroups; ++g) a.eip_group[(int64_t)g * a.n + p] = 1.0 / ipow(eps, (unsigned)T.gord[g]);
        }

        // ---- 2. Gram over the union basis ----
        double acc[NPP];
#pragma unroll
        for (int t = 0; t < NPP; ++t) acc[t] = 0.0;
        if (any_ok) {
            for (int c0 = 0; c0 < k; c0 += kCh) {
                int q = c0 + lane;
                const int cnt = min(kCh, k - c0);
                if (q < k) {
                    double o[DIM], u[DIM];
                    load_offset<DIM>(a, xp, a.cols[beg + q], o);
#pragma unroll
                    for (int d = 0; d < DIM; ++d) u[d] = o[d] / eps;
                    double E = cw_exp(-norm2<DIM>(o) / (2.0 * eps * eps));
                    double pw[kMaxDim][8];
                    powers<DIM, MAXE>(u, pw);
                    for (int j = 0; j < nu; ++j) Bs[lane * L.ldb + j] = E * mono<DIM, MAXE>(pw, T.uexp[j]);
                }
                __syncwarp();
                for (int r = 0; r < cnt; ++r) {
                    const double* row = Bs + r * L.ldb;
#pragma unroll
                    for (int t = 0; t < NPP; ++t)
                        if (t * 32 + lane < npairs) acc[t] = fma(row[pi[t]], row[pj[t]], acc[t]);
                }
                __syncwarp();
            }
#pragma unroll
            for (int t = 0; t < NPP; ++t)
                if (t * 32 + lane < npairs) Gs[t * 32 + lane] = acc[t];
            __syncwarp();
        }

        // ---- 3. per basis: column-pivoting QR solve ----
        for (int g = 0; g < ngroups; ++g) {
            if (gst[g] != ST_OK) continue;
            const int n = T.gn[g];
            const int nrhs = fast ? T.nout_rhs[g] : T.nterm_rhs[g];
            const int ncol = n + nrhs;
            // R = [A | b...]
            for (int e = lane; e < n * ncol; e += 32) {
                int i = e / ncol, j = e - i * ncol;
                double v;
                if (j < n) {
                    int ui = T.gidx[g][i], uj = T.gidx[g][j];
                    int lo = min(ui, uj), hi = max(ui, uj);
                    v = Gs[T.upair[lo][hi]];
                } else {
                    v = fast ? T.b_out[g][j - n][i] : T.b_term[g][j - n][i];
                }
                R[i * L.ldr + j] = v;
            }
            for (int i = lane; i < n; i += 32) perm[i] = i;
            __syncwarp();
            bool singular = false;
            for (int kk = 0; kk < n; ++kk) {
                // column norms of the trailing block, pivot = first largest
                double best = -1.0;
                int bidx = 0x7fffffff;
                for (int j = lane; j < n; j += 32) {
                    if (j < kk) continue;
                    double sn = 0.0;
                    for (int i = kk; i < n; ++i) sn = fma(R[i * L.ldr + j], R[i * L.ldr + j], sn);
                    if (sn > best) {
                        best = sn;
                        bidx = j;
                    }
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    double ob = __shfl_xor_sync(0xffffffffu, best, o);
                    int oi = __shfl_xor_sync(0xffffffffu, bidx, o);
                    if (ob > best || (ob == best && oi < bidx)) {
                        best = ob;
                        bidx = oi;
                    }
                }
                int piv = (bidx == 0x7fffffff) ? kk : bidx;
                // sigma = the pivot column's norm (NaN when all norms were NaN)
                double sigma;
                if (bidx == 0x7fffffff) {
                    double sn = 0.0;
                    for (int i = kk; i < n; ++i) sn = fma(R[i * L.ldr + kk], R[i * L.ldr + kk], sn);
                    sigma = sn;
                } else {
                    sigma = best;
                }
                if (!(sigma > 0.0)) {
                    singular = true;
                    break;
                }
                if (piv != kk) {
                    for (int i = lane; i < n; i += 32) {
                        double t0 = R[i * L.ldr + kk];
                        R[i * L.ldr + kk] = R[i * L.ldr + piv];
                        R[i * L.ldr + piv] = t0;
                    }
                    if (lane == 0) {
                        int t0 = perm[kk];
                        perm[kk] = perm[piv];
                        perm[piv] = t0;
                    }
                }
                __syncwarp();
                const double alpha = R[kk * L.ldr + kk];
                const double nr = sqrt(sigma);
                const double beta = (alpha >= 0.0) ? -nr : nr;
                const double den = alpha - beta;
                const double tau = (beta - alpha) / beta;
                __syncwarp();
                for (int i = kk + 1 + lane; i < n; i += 32) R[i * L.ldr + kk] = R[i * L.ldr + kk] / den;
                __syncwarp();
                if (lane == 0) R[kk * L.ldr + kk] = beta;
                for (int j = kk + 1 + lane; j < ncol; j += 32) {
                    double sv = R[kk * L.ldr + j];
                    for (int i = kk + 1; i < n; ++i) sv = fma(R[i * L.ldr + kk], R[i * L.ldr + j], sv);
                    sv = sv * tau;
                    R[kk * L.ldr + j] = R[kk * L.ldr + j] - sv;
                    for (int i = kk + 1; i < n; ++i) R[i * L.ldr + j] = fma(-sv, R[i * L.ldr + kk], R[i * L.ldr + j]);
                }
                __syncwarp();
            }
            if (singular) {
                gst[g] = ST_SINGULAR;
                __syncwarp();
                continue;
            }
            // back substitution, one right-hand side per lane
            double* Ag = Acoef + L.a_off[g];
            for (int r = lane; r < nrhs; r += 32) {
                for (int i = n - 1; i >= 0; --i) {
                    double sv = R[i * L.ldr + n + r];
                    for (int j = i + 1; j < n; ++j) sv = fma(-R[i * L.ldr + j], Z[j * kMaxRhs + r], sv);
                    Z[i * kMaxRhs + r] = sv / R[i * L.ldr + i];
                }
            }
            __syncwarp();
            for (int e = lane; e < n * nrhs; e += 32) {
                int i = e / nrhs, r = e - i * nrhs;
                Ag[perm[i] * kRhs + r] = Z[i * kMaxRhs + r];
            }
            __syncwarp();
        }

        // ---- 4. kernels ----
        double eipg[kMaxGroups];
#pragma unroll
        for (int g = 0; g < kMaxGroups; ++g) eipg[g] = (g < ngroups) ? 1.0 / ipow(eps, (unsigned)T.gord[g]) : 0.0;
        bool nonfinite = false;
        for (int c0 = 0; c0 < k; c0 += kCh) {
            int q = c0 + lane;
            if (q >= k) break;  // rows of this lane are done; no warp sync below
            double o[DIM], u[DIM];
            load_offset<DIM>(a, xp, a.cols[beg + q], o);
#pragma unroll
            for (int d = 0; d < DIM; ++d) u[d] = o[d] / eps;
            double pw[kMaxDim][8];
            powers<DIM, MAXE>(u, pw);
            const double ef = cw_exp(-norm2<DIM>(u));
            double wout[kMaxOutputs];
#pragma unroll
            for (int t = 0; t < kMaxOutputs; ++t) wout[t] = 0.0;
            for (int g = 0; g < ngroups; ++g) {
                const int n = T.gn[g];
                const int nrhs = fast ? T.nout_rhs[g] : T.nterm_rhs[g];
                const bool ok = (gst[g] == ST_OK);
                const double* Ag = Acoef + L.a_off[g];
                double res[kRhs];
#pragma unroll
                for (int r = 0; r < kRhs; ++r) res[r] = 0.0;
                if (ok) {
                    for (int i = 0; i < n; ++i) {
                        double v = mono<DIM, MAXE>(pw, T.uexp[T.gidx[g][i]]);
#pragma unroll
                        for (int r = 0; r < kRhs; ++r) {
                            if (r < nrhs) {
                                if (fast) {
                                    res[r] = fma(Ag[i * kRhs + r], v, res[r]);
                                } else {
                                    double t0 = Ag[i * kRhs + r] * v;
                                    t0 = t0 * ef;
                                    res[r] = res[r] + t0;
                                }
                            }
                        }
                    }
                }
                double eip = eipg[0];
#pragma unroll
                for (int t = 1; t < kMaxGroups; ++t)
                    if (t == g) eip = eipg[t];
#pragma unroll
                for (int r = 0; r < kRhs; ++r) {
                    if (r < nrhs) {
                        if (fast) {
                            double Kq = ok ? (res[r] * ef) : 0.0;
                            nonfinite |= !isfinite(Kq);
                            int o2 = T.out_of_rhs[g][r];
#pragma unroll
                            for (int t = 0; t < kMaxOutputs; ++t)
                                if (t == o2) wout[t] = wout[t] + Kq * eip;
                        } else {
                            double Kq = res[r];
                            nonfinite |= !isfinite(Kq);
                            int term = T.term_of_rhs[g][r];
                            if (st_terms) a.k_term[(int64_t)term * a.nnz + beg + q] = Kq;
                            int o2 = T.term_output[term];
#pragma unroll
                            for (int t = 0; t < kMaxOutputs; ++t)
                                if (t == o2) wout[t] = wout[t] + Kq * eip;
                        }
                    }
                }
            }
            for (int t = 0; t < noutputs; ++t) {
                if (a.w64) a.w64[(int64_t)t * a.nnz + beg + q] = wout[t];
                const float w32 = (float)wout[t];
                if (a.w32) a.w32[(int64_t)t * a.nnz + beg + q] = w32;
                if (a.r16)
                    reinterpret_cast<__nv_bfloat16*>(a.r16)[(int64_t)t * a.nnz + beg + q] =
                        __float2bfloat16_rn((float)(wout[t] - (double)w32));
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
                }
            }
        } else if (st_terms) {
            // failed groups: their term kernels are zero (written above as 0)
        }
        if (lane == 0) {
            int st = ST_OK;
            for (int g = 0; g < ngroups; ++g)
                if (st == ST_OK && gst[g] != ST_OK) st = gst[g];
            if (st == ST_OK && nonfinite) st = ST_NONFINITE;
            a.status[p] = st;
        }
        __syncwarp();
    }
}

template <int DIM, int MAXE, int NPP>
cudaError_t launch(const AsmArgs& a, const Layout& L, cudaStream_t s) {
    const int warps = (a.warps == 2 || a.warps == 8) ? a.warps : kWarps;
    size_t bytes = (size_t)L.words * sizeof(double) * warps;
    auto kern = assemble_kernel<DIM, MAXE, NPP>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, warps * 32, bytes);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    int64_t need = (a.n + warps - 1) / warps;
    int64_t grid = (int64_t)num_sms() * per_sm;
    if (grid > need) grid = need;
    if (grid < 1) grid = 1;
    kern<<<(unsigned)grid, warps * 32, bytes, s>>>(a, L);
    return cudaGetLastError();
}

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

template <int DIM>
cudaError_t dispatch(const AsmArgs& a, const AsmTables& h, const Layout& L, cudaStream_t s) {
    const int npp = (h.npairs + 31) / 32;
    if (h.maxexp <= 4) {
        if (npp <= 8) return launch<DIM, 4, 8>(a, L, s);
        return launch<DIM, 4, 40>(a, L, s);
    }
    if (npp <= 8) return launch<DIM, 8, 8>(a, L, s);
    return launch<DIM, 8, 40>(a, L, s);
}

}  // namespace

int64_t binning_tmp_elems(int64_t n, int maxk, int width) {
    const int64_t nb = maxk / (width > 0 ? width : 1) + 1;
    return nb + 1 + scan_tmp_elems(nb);
}

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
    Layout L{};
    L.ldb = h.nu | 1;
    L.nmax = 1;
    int rmax = 1;
    for (int g = 0; g < h.ngroups; ++g) {
        L.nmax = L.nmax > h.gn[g] ? L.nmax : h.gn[g];
        int r = (a.flags & DCPSE_ASSEMBLE_FAST_FLAG) ? h.nout_rhs[g] : h.nterm_rhs[g];
        rmax = rmax > r ? rmax : r;
    }
    L.ldr = (L.nmax + rmax) | 1;
    int off = 0;
    L.off_b = off;
    off += kCh * L.ldb;
    L.off_g = off;
    off += h.npairs;
    L.off_r = off;
    off += L.nmax * L.ldr;
    L.off_z = off;
    off += L.nmax * kMaxRhs;
    L.off_a = off;
    for (int g = 0; g < h.ngroups; ++g) {
        L.a_off[g] = off - L.off_a;
        off += h.gn[g] * kRhs;
    }
    L.off_perm = off;
    off += (L.nmax + 1) / 2;
    L.words = off + (off & 1);  // keep each warp's block 16-byte aligned
    if (h.dim == 3) return dispatch<3>(a, h, L, s);
    if (h.dim == 2) return dispatch<2>(a, h, L, s);
    return dispatch<1>(a, h, L, s);
}

}  // namespace dcpse
