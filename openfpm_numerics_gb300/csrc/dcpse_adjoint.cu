// dcpse_adjoint.cu -- vector-Jacobian products of the batched DC-PSE apply.
//
// The reference has no adjoint; these are the derivatives of its operator
// (src/DCPSE/Dcpse.hpp:690-809 assembly, :467-499 apply) with the
// neighbour lists held fixed.  With outputs y_o,p = sum_q W_o,pq (f_q - f_p):
//
//  * field VJP:   (dL/df)_q = sum_o [ sum_{p: q in N(p)} W_o,pq g_o,p
//                                     - g_o,q sum_r W_o,qr ]
//    through a transposed neighbour list (rows sorted by source particle, so
//    the sums run in a fixed order), built once per list;
//
//  * position VJP: for particle p and basis g, with c_q = f_q - f_p,
//    omega_q = exp(-|u_q|^2), u_q = x_pq / eps, v_q = m(u_q),
//    A = sum_q omega_q v_q v_q^T,  b~ = sum_o g_o,p b_o,g,
//    Phi = eps^-|alpha| s^T a~,  s = sum_q c_q omega_q v_q,  a~ = A^-1 b~:
//      lambda = A^-1 s,
//      dPhi/domega_q = e (v_q.a~)(c_q - v_q.lambda),
//      dPhi/dv_q     = e omega_q [ (c_q - v_q.lambda) a~ - (v_q.a~) lambda ],
//    chained through omega_q, v_q(u_q), u_q = x_pq/eps and
//    eps = sum_q |x_pq|_1 / (k HOverEpsilon), eps^-|alpha| into per-entry
//    contributions G_pq:  grad x_p += G_pq,  grad x_q -= G_pq.
//
// FP64 throughout; one warp per particle, neighbours in chunks of 32 rows;
// the per-particle systems are solved with the same column-pivoting QR as the
// assembly.
#include "dcpse_internal.h"

namespace dcpse {
namespace {

// ---------------------------------------------------- transposed CSR build --
__global__ void tcount_kernel(const int32_t* __restrict__ cols, int64_t nnz, int32_t* __restrict__ cnt) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nnz; j += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(&cnt[cols[j]], 1);
}

__global__ void tfill_kernel(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ cols, int64_t n,
                             int64_t* fill, int32_t* __restrict__ tsrc, int64_t* __restrict__ tidx) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
        for (int64_t j = rowptr[p]; j < rowptr[p + 1]; ++j) {
            unsigned long long slot = atomicAdd((unsigned long long*)&fill[cols[j]], 1ull);
            tsrc[slot] = (int32_t)p;
            tidx[slot] = j;
        }
    }
}

// warp per transposed row: order entries by source particle (distinct)
__global__ void tsort_kernel(const int64_t* __restrict__ trow, int64_t n, const int32_t* __restrict__ src_in,
                             const int64_t* __restrict__ idx_in, int32_t* __restrict__ src_out,
                             int64_t* __restrict__ idx_out) {
    const int lane = threadIdx.x & 31;
    const int64_t w0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t q = w0; q < n; q += nw) {
        const int64_t b = trow[q];
        const int k = (int)(trow[q + 1] - b);
        for (int i0 = 0; i0 < k; i0 += 32) {
            const int i = i0 + lane;
            const int32_t v = (i < k) ? src_in[b + i] : 0;
            int rank = 0;
            for (int j = 0; j < k; ++j) rank += (src_in[b + j] < v);
            if (i < k) {
                src_out[b + rank] = v;
                idx_out[b + rank] = idx_in[b + i];
            }
        }
    }
}

__global__ void rowsum_kernel(const int64_t* __restrict__ rowptr, int64_t n, int nout, const double* __restrict__ w64,
                              const float* __restrict__ w32, int64_t ws, double* __restrict__ rs) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
        for (int o = 0; o < nout; ++o) {
            double s = 0.0;
            for (int64_t j = rowptr[p]; j < rowptr[p + 1]; ++j)
                s = s + (w64 ? w64[(int64_t)o * ws + j] : (double)w32[(int64_t)o * ws + j]);
            rs[(int64_t)o * n + p] = s;
        }
    }
}

// (L^T g)_q in FP64, thread per transposed row, fixed order
__global__ void vjp_field_kernel(const int64_t* __restrict__ trow, const int32_t* __restrict__ tsrc,
                                 const int64_t* __restrict__ tidx, int64_t n, int nout, const double* __restrict__ w64,
                                 const float* __restrict__ w32, int64_t ws, const double* __restrict__ rs,
                                 const double* __restrict__ g, double* __restrict__ out) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        double acc = 0.0;
        for (int64_t t = trow[q]; t < trow[q + 1]; ++t) {
            const int64_t j = tidx[t];
            const int64_t p = tsrc[t];
            for (int o = 0; o < nout; ++o) {
                const double w = w64 ? w64[(int64_t)o * ws + j] : (double)w32[(int64_t)o * ws + j];
                acc = fma(w, g[(int64_t)o * n + p], acc);
            }
        }
        for (int o = 0; o < nout; ++o) acc = fma(-g[(int64_t)o * n + q], rs[(int64_t)o * n + q], acc);
        out[q] = acc;
    }
}

// (L^T g)_q on the sliced ELL layout of the transposed list (slices of 32
// rows stored entry-major, rows sorted by length within windows of 256; the
// weights of every output gathered into it): a row per thread, coalesced
// column and weight streams, the cotangents gathered per output.  Each row
// sums its entries in the CSR kernel's order (by source particle, outputs
// innermost) and subtracts the row-sum terms last, so the results are the
// CSR kernel's bit for bit; padding entries have weight 0 on the row itself.
// FP32 weights come widened to double at the layout's build (exact, as the
// CSR kernel's per-use conversion is, which runs at the FP64 rate here).
template <int NO>
__global__ void __launch_bounds__(256) vjp_field_sell_kernel(VjpSellArgs a) {
    const double* __restrict__ wt = a.w;
    const int lane = threadIdx.x & 31;
    constexpr int U = NO <= 2 ? 4 : 2;  // entries in flight per thread
    for (int64_t win = blockIdx.x; win < a.nwin; win += gridDim.x) {
        const int64_t s = win * 8 + (threadIdx.x >> 5);
        const int32_t row = a.srow[s * 32 + lane];
        if (row < 0) continue;
        const int64_t b = a.off[s];
        const int L = (int)((a.off[s + 1] - b) / 32);
        const int32_t* __restrict__ c = a.cols + b + lane;
        const double* __restrict__ w = wt + b + lane;
        double acc = 0.0;
        for (int j0 = 0; j0 < L; j0 += U) {
            int32_t q[U];
            double wv[U][NO], gv[U][NO];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int j = j0 + u;
                q[u] = j < L ? c[(int64_t)j * 32] : row;
#pragma unroll
                for (int o = 0; o < NO; ++o) wv[u][o] = j < L ? w[(int64_t)o * a.total + (int64_t)j * 32] : 0.0;
            }
#pragma unroll
            for (int u = 0; u < U; ++u)
#pragma unroll
                for (int o = 0; o < NO; ++o) gv[u][o] = a.g[(int64_t)o * a.n + q[u]];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                if (j0 + u < L) {
#pragma unroll
                    for (int o = 0; o < NO; ++o) acc = fma(wv[u][o], gv[u][o], acc);
                }
            }
        }
#pragma unroll
        for (int o = 0; o < NO; ++o) acc = fma(-a.g[(int64_t)o * a.n + row], a.rs[(int64_t)o * a.n + row], acc);
        a.out[row] = acc;
    }
}

// transposed weights of every output, as doubles: wt[o * nnz + t] =
// w[o * ws + tidx[t]] (FP32 weights widened, exactly)
template <typename T>
__global__ void transpose_outputs_kernel(const int64_t* __restrict__ tidx, int64_t nnz, int nout,
                                         const T* __restrict__ w, int64_t ws, double* __restrict__ wt) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nnz; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = tidx[t];
        for (int o = 0; o < nout; ++o) wt[(int64_t)o * nnz + t] = (double)w[(int64_t)o * ws + j];
    }
}

// ------------------------------------------------------------ position VJP --
constexpr int kWarps = 4;
constexpr int kCh = 32;

struct VjpLayout {
    int ldb;   // B chunk row stride: nu + 1 columns (the last is E c)
    int ldr;   // QR matrix stride (n + 2)
    int nmax;
    int off_b, off_g, off_r, off_z, off_ab, off_perm, words;
};

// powers u_d^t, t = 0..8, of one entry (computed once, then shared by all
// its monomials: the same products each monomial used to form itself)
template <int DIM>
__device__ __forceinline__ void powers(const double* u, double (&pw)[DIM][9]) {
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        pw[d][0] = 1.0;
#pragma unroll
        for (int t = 1; t < 9; ++t) pw[d][t] = pw[d][t - 1] * u[d];
    }
}

// m = prod_d u_d^e_d
template <int DIM>
__device__ __forceinline__ double mono(const double (&pw)[DIM][9], const unsigned char* e) {
    double m = 1.0;
#pragma unroll
    for (int d = 0; d < DIM; ++d) m *= pw[d][e[d]];
    return m;
}

// small integers as doubles (an int -> double conversion runs on the FP64
// pipe; the exponent is the same for all lanes, so the constant cache
// broadcasts it)
__constant__ double kSmallInt[9] = {0.0, 1.0, 2.0, 3.0, 4.0, 5.0, 6.0, 7.0, 8.0};

// dm_d = e_d u_d^(e_d - 1) prod_{d' != d} u_d'^e_d'
template <int DIM>
__device__ __forceinline__ void mono_grad(const double (&pw)[DIM][9], const unsigned char* e, double* dm) {
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        if (e[d] == 0) {
            dm[d] = 0.0;
            continue;
        }
        double r = kSmallInt[e[d]] * pw[d][e[d] - 1];
#pragma unroll
        for (int d2 = 0; d2 < DIM; ++d2)
            if (d2 != d) r *= pw[d2][e[d2]];
        dm[d] = r;
    }
}

template <int DIM, int NPP>
__global__ void __launch_bounds__(kWarps * 32) vjp_pos_kernel(VjpArgs a, VjpLayout L) {
    extern __shared__ double smem[];
    const AsmTables& T = *a.tab;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    double* S = smem + (size_t)wib * L.words;
    double* Bs = S + L.off_b;
    double* Gs = S + L.off_g;   // npairs Gram entries, then nu entries of s
    double* R = S + L.off_r;
    double* Z = S + L.off_z;
    double* AB = S + L.off_ab;  // per group: a~ [n] then lambda [n]
    int* perm = reinterpret_cast<int*>(S + L.off_perm);
    const int nu = T.nu, npairs = T.npairs, ngroups = T.ngroups;
    // pairs owned by this lane: Gram pairs, then (i, c) pairs for s
    const int nall = npairs + nu;
    int pi[NPP], pj[NPP];
#pragma unroll
    for (int t = 0; t < NPP; ++t) {
        const int e = t * 32 + lane;
        pi[t] = (e < npairs) ? T.pi[e] : (e < nall ? e - npairs : 0);
        pj[t] = (e < npairs) ? T.pj[e] : nu;
    }
    const int64_t gw = (int64_t)blockIdx.x * kWarps + wib, nw = (int64_t)gridDim.x * kWarps;
    for (int64_t p = gw; p < a.n; p += nw) {
        const int64_t beg = a.rowptr[p];
        const int k = (int)(a.rowptr[p + 1] - beg);
        double xp[DIM];
#pragma unroll
        for (int d = 0; d < DIM; ++d) xp[d] = a.pos[p * DIM + d];
        const double fp = a.f[p];
        // eps (as the assembly)
        double s = 0.0;
        for (int c0 = 0; c0 < k; c0 += kCh) {
            const int q = c0 + lane;
            double v = 0.0;
            if (q < k) {
                const int64_t qq = a.cols[beg + q];
                double acc = 0.0;
#pragma unroll
                for (int d = 0; d < DIM; ++d) acc = acc + fabs(offset1(a.geom, d, xp[d], a.pos[qq * DIM + d]));
                v = acc;
            }
            const int cnt = min(kCh, k - c0);
            for (int t = 0; t < kCh; ++t) {
                const double w = __shfl_sync(0xffffffffu, v, t);
                if (t < cnt) s = s + w;
            }
        }
        double eps = (s / (double)k) / a.h_over_eps;
        const bool fixed = a.eps_fixed != nullptr;
        if (fixed) eps = a.eps_fixed[p];
        bool ok = (eps > 0.0) && isfinite(eps);
        for (int g = 0; g < ngroups; ++g) ok = ok && (k >= T.gn[g]);
        if (!ok) {
            for (int q = lane; q < k; q += 32)
#pragma unroll
                for (int d = 0; d < DIM; ++d) a.gentry[(beg + q) * DIM + d] = 0.0;
            continue;
        }
        // one reciprocal of eps per particle (u = x_pq / eps as a product:
        // within an ulp of the assembly's quotient, well inside this
        // adjoint's tolerance)
        const double ieps = 1.0 / eps;
        // Gram + s
        double acc[NPP];
#pragma unroll
        for (int t = 0; t < NPP; ++t) acc[t] = 0.0;
        for (int c0 = 0; c0 < k; c0 += kCh) {
            const int q = c0 + lane;
            const int cnt = min(kCh, k - c0);
            if (q < k) {
                const int64_t qq = a.cols[beg + q];
                double o[DIM], u[DIM];
#pragma unroll
                for (int d = 0; d < DIM; ++d) {
                    o[d] = offset1(a.geom, d, xp[d], a.pos[qq * DIM + d]);
                    u[d] = o[d] * ieps;
                }
                const double E = exp(-0.5 * norm2<DIM>(u));  // E^2 = omega
                double pw[DIM][9];
                powers<DIM>(u, pw);
                for (int j = 0; j < nu; ++j) Bs[lane * L.ldb + j] = E * mono<DIM>(pw, T.uexp[j]);
                Bs[lane * L.ldb + nu] = E * (a.f[qq] - fp);
            }
            __syncwarp();
            for (int r = 0; r < cnt; ++r) {
                const double* row = Bs + r * L.ldb;
#pragma unroll
                for (int t = 0; t < NPP; ++t)
                    if (t * 32 + lane < nall) acc[t] = fma(row[pi[t]], row[pj[t]], acc[t]);
            }
            __syncwarp();
        }
#pragma unroll
        for (int t = 0; t < NPP; ++t)
            if (t * 32 + lane < nall) Gs[t * 32 + lane] = acc[t];
        __syncwarp();
        // per group: solve for a~ (b~ = sum_o g_o b_o) and lambda (s)
        double Dsc = 0.0;  // d Phi / d eps from eps^-|alpha|
        bool singular = false;
        for (int g = 0; g < ngroups && !singular; ++g) {
            const int n = T.gn[g];
            const int ncol = n + 2;
            for (int e = lane; e < n * ncol; e += 32) {
                const int i = e / ncol, j = e - i * ncol;
                const int ui = T.gidx[g][i];
                double v;
                if (j < n) {
                    const int uj = T.gidx[g][j];
                    v = Gs[T.upair[min(ui, uj)][max(ui, uj)]];
                } else if (j == n) {
                    v = 0.0;
                    for (int r = 0; r < T.nout_rhs[g]; ++r) v += a.gbar[(int64_t)T.out_of_rhs[g][r] * a.n + p] * T.b_out[g][r][i];
                } else {
                    v = Gs[npairs + ui];
                }
                R[i * L.ldr + j] = v;
            }
            for (int i = lane; i < n; i += 32) perm[i] = i;
            __syncwarp();
            for (int kk = 0; kk < n; ++kk) {
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
                    const double ob = __shfl_xor_sync(0xffffffffu, best, o);
                    const int oi = __shfl_xor_sync(0xffffffffu, bidx, o);
                    if (ob > best || (ob == best && oi < bidx)) {
                        best = ob;
                        bidx = oi;
                    }
                }
                if (!(best > 0.0)) {
                    singular = true;
                    break;
                }
                const int piv = bidx;
                if (piv != kk) {
                    for (int i = lane; i < n; i += 32) {
                        const double t0 = R[i * L.ldr + kk];
                        R[i * L.ldr + kk] = R[i * L.ldr + piv];
                        R[i * L.ldr + piv] = t0;
                    }
                    if (lane == 0) {
                        const int t0 = perm[kk];
                        perm[kk] = perm[piv];
                        perm[piv] = t0;
                    }
                }
                __syncwarp();
                const double alpha = R[kk * L.ldr + kk];
                const double nr = sqrt(best);
                const double beta = (alpha >= 0.0) ? -nr : nr;
                const double den = alpha - beta, tau = (beta - alpha) / beta;
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
            if (singular) break;
            for (int r = lane; r < 2; r += 32) {
                for (int i = n - 1; i >= 0; --i) {
                    double sv = R[i * L.ldr + n + r];
                    for (int j = i + 1; j < n; ++j) sv = fma(-R[i * L.ldr + j], Z[j * 2 + r], sv);
                    Z[i * 2 + r] = sv / R[i * L.ldr + i];
                }
            }
            __syncwarp();
            double* ab = AB + g * 2 * L.nmax;
            for (int i = lane; i < n; i += 32) {
                ab[perm[i]] = Z[i * 2];
                ab[L.nmax + perm[i]] = Z[i * 2 + 1];
            }
            __syncwarp();
            // eps^-|alpha| term: d/deps of e = -m e / eps, times s^T a~
            const double ee = 1.0 / ipow(eps, (unsigned)T.gord[g]);
            double sa = 0.0;
            for (int i = 0; i < n; ++i) sa += Gs[npairs + T.gidx[g][i]] * ab[i];
            Dsc += -(double)T.gord[g] * ee * sa / eps;
        }
        if (singular) {
            for (int q = lane; q < k; q += 32)
#pragma unroll
                for (int d = 0; d < DIM; ++d) a.gentry[(beg + q) * DIM + d] = 0.0;
            continue;
        }
        // per-entry chain rule: the first pass stores gu / eps and sums
        // gu_q.u_q, which the eps term needs; the second adds that term
        double eeg[kMaxGroups];
#pragma unroll
        for (int g = 0; g < kMaxGroups; ++g) eeg[g] = g < ngroups ? 1.0 / ipow(eps, (unsigned)T.gord[g]) : 0.0;
        double gsum = 0.0;
        for (int c0 = 0; c0 < k; c0 += kCh) {
            const int q = c0 + lane;
            if (q >= k) break;
            const int64_t qq = a.cols[beg + q];
            double u[DIM], gu[DIM];
#pragma unroll
            for (int d = 0; d < DIM; ++d) {
                u[d] = offset1(a.geom, d, xp[d], a.pos[qq * DIM + d]) * ieps;
                gu[d] = 0.0;
            }
            const double om = exp(-norm2<DIM>(u));
            const double cq = a.f[qq] - fp;
            double pw[DIM][9];
            powers<DIM>(u, pw);
            for (int g = 0; g < ngroups; ++g) {
                const int n = T.gn[g];
                const double* at = AB + g * 2 * L.nmax;
                const double* lm = at + L.nmax;
                double ee = eeg[0];
#pragma unroll
                for (int t = 1; t < kMaxGroups; ++t)
                    if (t == g) ee = eeg[t];
                double va = 0.0, vl = 0.0;
                for (int i = 0; i < n; ++i) {
                    const double vi = mono<DIM>(pw, T.uexp[T.gidx[g][i]]);
                    va = fma(vi, at[i], va);
                    vl = fma(vi, lm[i], vl);
                }
                const double r = cq - vl;
                const double alpha_q = ee * va * r;
                const double ga = alpha_q * (-2.0 * om);
#pragma unroll
                for (int d = 0; d < DIM; ++d) gu[d] = fma(ga, u[d], gu[d]);
                const double eo = ee * om;
                for (int i = 0; i < n; ++i) {
                    double dvi[DIM];
                    mono_grad<DIM>(pw, T.uexp[T.gidx[g][i]], dvi);
                    const double beta_i = eo * fma(r, at[i], -va * lm[i]);
#pragma unroll
                    for (int d = 0; d < DIM; ++d) gu[d] = fma(beta_i, dvi[d], gu[d]);
                }
            }
            double t = 0.0;
#pragma unroll
            for (int d = 0; d < DIM; ++d) {
                t = fma(gu[d], u[d], t);
                a.gentry[(beg + q) * DIM + d] = gu[d] * ieps;
            }
            gsum += t;
        }
        for (int o = 16; o > 0; o >>= 1) gsum += __shfl_xor_sync(0xffffffffu, gsum, o);
        // (with a fixed eps the term is zero; adding it keeps the sign of
        // zero entries as the fused expression gu / eps + dd sg gave it)
        const double dd = fixed ? 0.0 : (Dsc - gsum / eps) / ((double)k * a.h_over_eps);
        for (int q = lane; q < k; q += 32) {
            const int64_t qq = a.cols[beg + q];
#pragma unroll
            for (int d = 0; d < DIM; ++d) {
                const double o = offset1(a.geom, d, xp[d], a.pos[qq * DIM + d]);
                const double sg = (o > 0.0) ? 1.0 : ((o < 0.0) ? -1.0 : 0.0);
                a.gentry[(beg + q) * DIM + d] = a.gentry[(beg + q) * DIM + d] + dd * sg;
            }
        }
    }
}

// grad x_i = sum_{j in row i} G_j - sum_{entries pointing at i} G
__global__ void vjp_pos_gather_kernel(const int64_t* __restrict__ rowptr, const int64_t* __restrict__ trow,
                                      const int64_t* __restrict__ tidx, int64_t n, int dim,
                                      const double* __restrict__ G, double* __restrict__ grad) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        for (int d = 0; d < dim; ++d) {
            double s = 0.0;
            for (int64_t j = rowptr[i]; j < rowptr[i + 1]; ++j) s += G[j * dim + d];
            for (int64_t t = trow[i]; t < trow[i + 1]; ++t) s -= G[tidx[t] * dim + d];
            grad[i * dim + d] = s;
        }
    }
}

int grid_for(int64_t items) {
    int64_t g = (items + 255) / 256, cap = (int64_t)num_sms() * 8;
    return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

template <int DIM, int NPP>
cudaError_t launch_vjp(const VjpArgs& a, const VjpLayout& L, cudaStream_t s) {
    size_t bytes = (size_t)L.words * sizeof(double) * kWarps;
    auto kern = vjp_pos_kernel<DIM, NPP>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kWarps * 32, bytes);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    int64_t need = (a.n + kWarps - 1) / kWarps, grid = (int64_t)num_sms() * per_sm;
    if (grid > need) grid = need;
    if (grid < 1) grid = 1;
    kern<<<(unsigned)grid, kWarps * 32, bytes, s>>>(a, L);
    return cudaGetLastError();
}

}  // namespace

cudaError_t build_transpose(const int64_t* rowptr, const int32_t* cols, int64_t n, int64_t nnz, int32_t* cnt,
                            int64_t* trow, int64_t* fill, int32_t* tsrc_tmp, int64_t* tidx_tmp, int32_t* tsrc,
                            int64_t* tidx, int64_t* scan_tmp, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(cnt, 0, sizeof(int32_t) * (n > 0 ? n : 1), s);
    if (e != cudaSuccess || n == 0) return e;
    if (nnz > 0) tcount_kernel<<<grid_for(nnz), 256, 0, s>>>(cols, nnz, cnt);
    e = exclusive_scan_i32(cnt, n, trow, scan_tmp, s);
    if (e != cudaSuccess) return e;
    e = cudaMemcpyAsync(fill, trow, sizeof(int64_t) * n, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return e;
    tfill_kernel<<<grid_for(n), 256, 0, s>>>(rowptr, cols, n, fill, tsrc_tmp, tidx_tmp);
    tsort_kernel<<<grid_for(n * 32), 256, 0, s>>>(trow, n, tsrc_tmp, tidx_tmp, tsrc, tidx);
    return cudaGetLastError();
}

cudaError_t row_sums(const int64_t* rowptr, int64_t n, int nout, const double* w64, const float* w32, int64_t ws,
                     double* rs, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    rowsum_kernel<<<grid_for(n), 256, 0, s>>>(rowptr, n, nout, w64, w32, ws, rs);
    return cudaGetLastError();
}

cudaError_t vjp_field(const int64_t* trow, const int32_t* tsrc, const int64_t* tidx, int64_t n, int nout,
                      const double* w64, const float* w32, int64_t ws, const double* rs, const double* g, double* out,
                      cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    vjp_field_kernel<<<grid_for(n), 256, 0, s>>>(trow, tsrc, tidx, n, nout, w64, w32, ws, rs, g, out);
    return cudaGetLastError();
}

cudaError_t vjp_field_sell(const VjpSellArgs& a, int nout, cudaStream_t s) {
    if (a.nwin == 0) return cudaSuccess;
    if (a.nwin > 0x7fffffff) return cudaErrorInvalidValue;
    const unsigned grid = (unsigned)a.nwin;
    switch (nout) {
#define DCPSE_VJPS_CASE(NO)                                       \
    case NO:                                                      \
        vjp_field_sell_kernel<NO><<<grid, 256, 0, s>>>(a);        \
        break;
        DCPSE_VJPS_CASE(1)
        DCPSE_VJPS_CASE(2)
        DCPSE_VJPS_CASE(3)
        DCPSE_VJPS_CASE(4)
        DCPSE_VJPS_CASE(5)
        DCPSE_VJPS_CASE(6)
        DCPSE_VJPS_CASE(7)
        DCPSE_VJPS_CASE(8)
#undef DCPSE_VJPS_CASE
        default:
            return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t transpose_outputs(const int64_t* tidx, int64_t nnz, int nout, const double* w64, const float* w32,
                              int64_t ws, double* wt, cudaStream_t s) {
    if (nnz == 0) return cudaSuccess;
    if (w64)
        transpose_outputs_kernel<double><<<grid_for(nnz), 256, 0, s>>>(tidx, nnz, nout, w64, ws, wt);
    else
        transpose_outputs_kernel<float><<<grid_for(nnz), 256, 0, s>>>(tidx, nnz, nout, w32, ws, wt);
    return cudaGetLastError();
}

cudaError_t vjp_positions(const VjpArgs& a, const AsmTables& h, const int64_t* trow, const int64_t* tidx, double* grad,
                          cudaStream_t s) {
    if (a.n == 0) return cudaSuccess;
    VjpLayout L{};
    L.ldb = (h.nu + 1) | 1;
    L.nmax = 1;
    for (int g = 0; g < h.ngroups; ++g) L.nmax = L.nmax > h.gn[g] ? L.nmax : h.gn[g];
    L.ldr = (L.nmax + 2) | 1;
    int off = 0;
    L.off_b = off;
    off += kCh * L.ldb;
    L.off_g = off;
    off += h.npairs + h.nu;
    L.off_r = off;
    off += L.nmax * L.ldr;
    L.off_z = off;
    off += L.nmax * 2;
    L.off_ab = off;
    off += h.ngroups * 2 * L.nmax;
    L.off_perm = off;
    off += (L.nmax + 1) / 2;
    L.words = off + (off & 1);
    const int npp = (h.npairs + h.nu + 31) / 32;
    cudaError_t e;
    if (h.dim == 3)
        e = npp <= 8 ? launch_vjp<3, 8>(a, L, s) : launch_vjp<3, 40>(a, L, s);
    else if (h.dim == 2)
        e = npp <= 8 ? launch_vjp<2, 8>(a, L, s) : launch_vjp<2, 40>(a, L, s);
    else
        e = npp <= 8 ? launch_vjp<1, 8>(a, L, s) : launch_vjp<1, 40>(a, L, s);
    if (e != cudaSuccess) return e;
    vjp_pos_gather_kernel<<<grid_for(a.n), 256, 0, s>>>(a.rowptr, trow, tidx, a.n, h.dim, a.gentry, grad);
    return cudaGetLastError();
}

}  // namespace dcpse
