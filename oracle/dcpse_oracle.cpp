// dcpse_oracle.cpp -- CPU FP64 restatement of openfpm_numerics' DC-PSE path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA product in
// openfpm_numerics_gb300/csrc: only tests/, __graft_entry__.smoke() and the
// cpu_baseline / reference leg of bench.py load it.  Nothing in the product
// links or calls it.
//
// What it restates (paths relative to the openfpm_numerics source tree):
//   basis        src/DCPSE/MonomialBasis.hpp:114-157 (generateBasis)
//   monomials    src/DCPSE/Monomial.hpp:146-174 (evaluate, getDerivative)
//   rhs          src/DCPSE/DcpseRhs.hpp:26-60
//   eps          src/DCPSE/Vandermonde.hpp:63-116 (computeEps, initialize)
//   V            src/DCPSE/Vandermonde.hpp:36-49, VandermondeRowBuilder.hpp:24-35
//   E (dense)    src/DCPSE/DcpseDiagonalScalingMatrix.hpp:21-41
//   B, A, solve  src/DCPSE/Dcpse.hpp:745-766
//   kernels      src/DCPSE/Dcpse.hpp:768-782, 798-809
//   apply        src/DCPSE/Dcpse.hpp:467-499 (bulk) and 560-603 (per key)
//
// The structure of the reference is kept on purpose: the diagonal scaling
// matrix E is a dense k x k matrix, B = E*V is a dense product, and every
// reference Dcpse object (e.g. each of the dim components of a Laplacian) is
// assembled on its own.
//
// Floating-point contract.  Built with -ffp-contract=off; every fused
// multiply-add below is an explicit std::fma.  Together with the exp below
// (identical operation sequence on the GPU) this fixes the rounding of every
// step, so the CUDA assembly can be compared with this file bit for bit.
//
// Third-party arithmetic that the reference delegates and that is absent here:
//  * Eigen3 ColPivHouseholderQR (Dcpse.hpp:766; Eigen version not pinned by
//    the reference).  Restated as Businger & Golub (1965), "Linear least
//    squares solutions by Householder transformations", Numer. Math. 7:
//    Householder QR with column pivoting on the largest remaining column
//    norm, norms recomputed at every step (no downdating).
//  * openfpm_data openfpm::math::intpowlog (Monomial.hpp:153, Dcpse.hpp:743):
//    restated as exponentiation by squaring.
//  * libm exp: restated as Cody & Waite argument reduction (Cody & Waite,
//    "Software Manual for the Elementary Functions", 1980) with the degree-13
//    Taylor polynomial of exp on |r| <= ln2/2, evaluated by Horner's rule.
//  * openfpm_data VerletList (order of neighbours): the neighbour set is the
//    predicate |x_p - x_q|^2 < rCut^2, q != p (VL_SKIP_REF_PART); the order is
//    ascending support index.  The reference's tests do not pin the order.
//
// Parity status: the reference cannot be compiled here (openfpm_data,
// openfpm_pdata, Eigen, Boost and MPI are absent), and its tests pin no
// DC-PSE weights.  This restatement is pinned against the reference's
// known-answer unit tests (basis sets, derivative scalars, row patterns, rhs
// signs) and its analytic error bars (tests/test_oracle_*.py).

#include <algorithm>
#include <map>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <thread>
#include <vector>

namespace {

// ---------------------------------------------------------------- exp -----
// ln2 split so that k*LN2_HI is exact for |k| < 2^21 (LN2_HI has 32
// significant bits); LN2_LO = ln2 - LN2_HI rounded to double.
const double LN2_HI = 0x1.62e42ff000000p-1;
const double LN2_LO = -0x1.718432a1b0e26p-35;
const double INV_LN2 = 0x1.71547652b82fep+0;
// 1/j! rounded to nearest, j = 0..13
const double TC[14] = {
    0x1.0000000000000p+0, 0x1.0000000000000p+0, 0x1.0000000000000p-1,
    0x1.5555555555555p-3, 0x1.5555555555555p-5, 0x1.1111111111111p-7,
    0x1.6c16c16c16c17p-10, 0x1.a01a01a01a01ap-13, 0x1.a01a01a01a01ap-16,
    0x1.71de3a556c734p-19, 0x1.27e4fb7789f5cp-22, 0x1.ae64567f544e4p-26,
    0x1.1eed8eff8d898p-29, 0x1.6124613a86d09p-33};

inline double pow2i(int k) {
    // 2^k for -1022 <= k <= 1023 built from the exponent field
    uint64_t bits = (uint64_t)(k + 1023) << 52;
    double r;
    std::memcpy(&r, &bits, sizeof r);
    return r;
}

inline double cw_exp(double x) {
    if (x != x) return x;
    if (x > 709.0) return std::numeric_limits<double>::infinity();
    if (x < -745.0) return 0.0;
    double kd = std::nearbyint(x * INV_LN2);
    double r = std::fma(-kd, LN2_HI, x);
    r = std::fma(-kd, LN2_LO, r);
    double p = TC[13];
    for (int j = 12; j >= 0; --j) p = std::fma(p, r, TC[j]);
    int k = (int)kd;
    if (k < -1022) {
        p = p * pow2i(-1022);
        k = k + 1022;
    }
    return p * pow2i(k);
}

// ------------------------------------------------------------ monomials ---
inline double ipow(double x, unsigned e) {
    if (e == 0) return 1.0;
    if (e == 1) return x;
    double h = ipow(x, e / 2);
    double r = h * h;
    if (e & 1u) r = r * x;
    return r;
}

struct Basis {
    int dim = 0;
    int n = 0;
    std::vector<unsigned> exps;     // n x dim
    std::vector<unsigned> scalars;  // n
};

// MonomialBasis.hpp:114-157.  Grid [0, lim)^dim visited with index 0 fastest
// (openfpm grid iterators advance dimension 0 first); kept when
// alphaMin <= |m| < lim, lim = |alpha| + r, alphaMin = 1 for even |alpha| > 0.
Basis make_basis(int dim, const unsigned* sig, unsigned r) {
    Basis b;
    b.dim = dim;
    unsigned msum = 0;
    for (int d = 0; d < dim; ++d) msum += sig[d];
    unsigned lim = msum + r;
    unsigned amin = (msum % 2 == 0) ? 1u : 0u;
    if (msum == 0) amin = 0;
    long total = 1;
    for (int d = 0; d < dim; ++d) total *= (long)lim;
    for (long lin = 0; lin < total; ++lin) {
        unsigned e[3] = {0, 0, 0};
        long t = lin;
        unsigned o = 0;
        for (int d = 0; d < dim; ++d) {
            e[d] = (unsigned)(t % lim);
            t /= lim;
            o += e[d];
        }
        if (o < lim && o >= amin) {
            for (int d = 0; d < dim; ++d) b.exps.push_back(e[d]);
            b.scalars.push_back(1u);
            b.n++;
        }
    }
    return b;
}

// Monomial.hpp:146-156
inline double mono_eval(int dim, const unsigned* e, unsigned scalar, const double* x) {
    double res = (double)scalar;
    for (int d = 0; d < dim; ++d) res = res * ipow(x[d], e[d]);
    return res;
}

// Monomial.hpp:158-174
void mono_deriv(int dim, const unsigned* e, unsigned scalar, const unsigned* dord,
                unsigned* oe, unsigned* os) {
    unsigned s = scalar;
    for (int d = 0; d < dim; ++d) {
        unsigned orig = e[d];
        int target = (int)orig - (int)dord[d];
        for (int k = (int)orig; k > target && k >= 0; --k) s *= (unsigned)k;
        oe[d] = (unsigned)std::max(target, 0);
    }
    *os = s;
}

// DcpseRhs.hpp:26-60: b_i = sign * (D^alpha m_i)(0), sign = +1 for even |alpha|
void make_rhs(const Basis& B, const unsigned* sig, double* b) {
    unsigned ord = 0;
    for (int d = 0; d < B.dim; ++d) ord += sig[d];
    int sign = (ord % 2 == 0) ? 1 : -1;
    const double zero[3] = {0.0, 0.0, 0.0};
    for (int i = 0; i < B.n; ++i) {
        unsigned de[3], ds;
        mono_deriv(B.dim, &B.exps[i * B.dim], B.scalars[i], sig, de, &ds);
        b[i] = sign * mono_eval(B.dim, de, ds, zero);
    }
}

// ------------------------------------------------------------- geometry ---
struct Geom {
    int dim = 0;
    double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0}, L[3] = {0, 0, 0};
    int per[3] = {0, 0, 0};
};

Geom make_geom(int dim, const double* lo, const double* hi, const int* per) {
    Geom g;
    g.dim = dim;
    for (int d = 0; d < dim; ++d) {
        g.lo[d] = lo ? lo[d] : 0.0;
        g.hi[d] = hi ? hi[d] : 0.0;
        g.L[d] = g.hi[d] - g.lo[d];
        g.per[d] = (per && lo && hi) ? per[d] : 0;
    }
    return g;
}

// x_p - x_q, with the minimum image along periodic axes
inline double offset1(const Geom& g, int d, double a, double b) {
    double o = a - b;
    if (g.per[d]) {
        double L = g.L[d];
        double h = 0.5 * L;
        if (o > h)
            o = o - L;
        else if (o < -h)
            o = o + L;
    }
    return o;
}

inline double norm2(int dim, const double* x) {
    double s = x[0] * x[0];
    for (int d = 1; d < dim; ++d) s = s + x[d] * x[d];
    return s;
}

// ------------------------------------------------------------ threading ---
template <class F>
void parallel_for(int64_t n, int nthreads, F f) {
    if (nthreads <= 1 || n < 2 * nthreads) {
        f(0, n);
        return;
    }
    std::vector<std::thread> th;
    int64_t chunk = (n + nthreads - 1) / nthreads;
    for (int t = 0; t < nthreads; ++t) {
        int64_t b = t * chunk, e = std::min(n, b + chunk);
        if (b >= e) break;
        th.emplace_back([=] { f(b, e); });
    }
    for (auto& t : th) t.join();
}

// ------------------------------------------------------------- CPQR -------
// Businger-Golub Householder QR with column pivoting, solving A a = b for
// nrhs right-hand sides.  R is n x n row-major, C is n x nrhs row-major.
// Returns false when a pivot column has zero norm (singular system).
bool cpqr_solve(int n, int nrhs, double* R, double* C, double* out /* n x nrhs */) {
    std::vector<int> perm(n);
    std::vector<double> nrm(n);
    for (int i = 0; i < n; ++i) perm[i] = i;
    for (int k = 0; k < n; ++k) {
        for (int j = k; j < n; ++j) {
            double s = 0.0;
            for (int i = k; i < n; ++i) s = std::fma(R[i * n + j], R[i * n + j], s);
            nrm[j] = s;
        }
        int piv = k;
        double best = -1.0;
        for (int j = k; j < n; ++j)
            if (nrm[j] > best) {
                best = nrm[j];
                piv = j;
            }
        if (piv != k) {
            for (int i = 0; i < n; ++i) std::swap(R[i * n + k], R[i * n + piv]);
            std::swap(perm[k], perm[piv]);
        }
        double sigma = nrm[piv];
        if (!(sigma > 0.0)) return false;
        double alpha = R[k * n + k];
        double nr = std::sqrt(sigma);
        double beta = (alpha >= 0.0) ? -nr : nr;
        double den = alpha - beta;
        for (int i = k + 1; i < n; ++i) R[i * n + k] = R[i * n + k] / den;
        double tau = (beta - alpha) / beta;
        R[k * n + k] = beta;
        for (int j = k + 1; j < n + nrhs; ++j) {
            double* col;
            int ld;
            if (j < n) {
                col = R + j;
                ld = n;
            } else {
                col = C + (j - n);
                ld = nrhs;
            }
            double s = col[k * ld];
            for (int i = k + 1; i < n; ++i) s = std::fma(R[i * n + k], col[i * ld], s);
            s = s * tau;
            col[k * ld] = col[k * ld] - s;
            for (int i = k + 1; i < n; ++i) col[i * ld] = std::fma(-s, R[i * n + k], col[i * ld]);
        }
    }
    std::vector<double> z(n);
    for (int r = 0; r < nrhs; ++r) {
        for (int i = n - 1; i >= 0; --i) {
            double s = C[i * nrhs + r];
            for (int j = i + 1; j < n; ++j) s = std::fma(-R[i * n + j], z[j], s);
            z[i] = s / R[i * n + i];
        }
        for (int i = 0; i < n; ++i) out[perm[i] * nrhs + r] = z[i];
    }
    return true;
}

enum { ST_OK = 0, ST_TOO_FEW = 1, ST_BAD_EPS = 2, ST_SINGULAR = 3, ST_NONFINITE = 4 };

struct AsmCtx {
    int dim;
    const double* pd;
    const double* ps;
    const int64_t* rowptr;
    const int32_t* cols;
    Geom g;
    Basis B;
    std::vector<double> b;
    unsigned ord;
    double hoe;
    const double* eps_fixed;  // optional per-particle eps override (extension)
    bool exact_gram = false;  // A = B^T B summed in double-double, rounded once (test aid)
};

// Dcpse.hpp:716-785 for one domain particle p.
int assemble_one(const AsmCtx& c, int64_t p, double* K, double& eps_out, double& eip_out) {
    const int dim = c.dim;
    const int64_t beg = c.rowptr[p];
    const int k = (int)(c.rowptr[p + 1] - beg);
    const int n = c.B.n;
    std::vector<double> X((size_t)k * dim);
    for (int q = 0; q < k; ++q) {
        const double* xq = c.ps + (size_t)c.cols[beg + q] * dim;
        for (int d = 0; d < dim; ++d) X[(size_t)q * dim + d] = offset1(c.g, d, c.pd[(size_t)p * dim + d], xq[d]);
    }
    for (int q = 0; q < k; ++q) K[q] = 0.0;
    // Vandermonde.hpp:63-81 (computeEps)
    double s = 0.0;
    for (int q = 0; q < k; ++q) {
        double a = 0.0;
        for (int d = 0; d < dim; ++d) a = a + std::fabs(X[(size_t)q * dim + d]);
        s = s + a;
    }
    s = s / (double)k;
    double eps = s / c.hoe;
    if (c.eps_fixed) eps = c.eps_fixed[p];
    eps_out = eps;
    eip_out = 1.0 / ipow(eps, c.ord);  // Dcpse.hpp:743
    if (k < n) return ST_TOO_FEW;       // Vandermonde.hpp:109-112
    if (!(eps > 0.0) || !std::isfinite(eps)) return ST_BAD_EPS;
    // V = m_j(x_pq / eps)   (Vandermonde.hpp:36-49)
    std::vector<double> U((size_t)k * dim), V((size_t)k * n);
    for (int q = 0; q < k; ++q) {
        for (int d = 0; d < dim; ++d) U[(size_t)q * dim + d] = X[(size_t)q * dim + d] / eps;
        for (int j = 0; j < n; ++j)
            V[(size_t)q * n + j] = mono_eval(dim, &c.B.exps[j * dim], c.B.scalars[j], &U[(size_t)q * dim]);
    }
    // dense E (DcpseDiagonalScalingMatrix.hpp:21-41)
    std::vector<double> E((size_t)k * k, 0.0);
    for (int q = 0; q < k; ++q)
        E[(size_t)q * k + q] = cw_exp(-norm2(dim, &X[(size_t)q * dim]) / (2.0 * eps * eps));
    // B = E V (Dcpse.hpp:755)
    std::vector<double> Bm((size_t)k * n);
    for (int q = 0; q < k; ++q)
        for (int j = 0; j < n; ++j) {
            double acc = 0.0;
            for (int r = 0; r < k; ++r) acc = acc + E[(size_t)q * k + r] * V[(size_t)r * n + j];
            Bm[(size_t)q * n + j] = acc;
        }
    // A = B^T B (Dcpse.hpp:757)
    std::vector<double> A((size_t)n * n);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            double acc = 0.0;
            if (!c.exact_gram) {
                for (int q = 0; q < k; ++q) acc = std::fma(Bm[(size_t)q * n + i], Bm[(size_t)q * n + j], acc);
            } else {
                // the same sum with error-free products (fma) and additions
                // (Knuth's two-sum) carried in a second double: the
                // correctly rounded Gram entry but for rare ties, against
                // which rounding orders of the Gram can be judged
                double lo = 0.0;
                for (int q = 0; q < k; ++q) {
                    const double x = Bm[(size_t)q * n + i], y = Bm[(size_t)q * n + j];
                    const double pr = x * y, pe = std::fma(x, y, -pr);
                    const double sm = acc + pr, bb = sm - acc;
                    const double se = (acc - (sm - bb)) + (pr - bb);
                    acc = sm;
                    lo = lo + (se + pe);
                }
                acc = acc + lo;
            }
            A[(size_t)i * n + j] = acc;
        }
    // a = A^-1 b (Dcpse.hpp:760-766)
    std::vector<double> rhs(c.b), a(n);
    if (!cpqr_solve(n, 1, A.data(), rhs.data(), a.data())) return ST_SINGULAR;
    // kernels (Dcpse.hpp:768-782, computeKernel 798-809)
    for (int q = 0; q < k; ++q) {
        const double* u = &U[(size_t)q * dim];
        double ef = cw_exp(-norm2(dim, u));
        double res = 0.0;
        for (int i = 0; i < n; ++i) {
            double t = a[i] * V[(size_t)q * n + i];
            t = t * ef;
            res = res + t;
        }
        K[q] = res;
    }
    for (int q = 0; q < k; ++q)
        if (!std::isfinite(K[q])) {
            for (int r = 0; r < k; ++r) K[r] = 0.0;
            return ST_NONFINITE;
        }
    return ST_OK;
}

// The reference's GPU assembly, Dcpse_gpu (src/DCPSE/Dcpse.cuh:776-842,
// 844-875), for one domain particle p.  Same basis and rhs as the CPU Dcpse;
// what differs:
//  * eps = 2 * (sum over neighbours and axes of |x_pq,d|) / k, one running
//    sum (FACTOR = 2, :799-807); epsInvPow = 1 / pow(eps, |alpha|);
//  * V_qj = m_j(x_pq) / pow(eps, |m_j|), monomials by pow per axis
//    (Monomial.cuh:156-163); E_qq = exp(-|x_pq|^2 / (2 eps^2));
//  * A = B^T B by plain sums, then LU WITHOUT pivoting (cublas<t>getrfBatched
//    with a null pivot array, Dcpse.cuh:683) and the two triangular solves
//    (lower unit, upper non-unit, :690-691), here as Doolittle elimination in
//    textbook order;
//  * K_q = sum_i a_i m_i(x_pq / eps) exp(-|x_pq / eps|^2), the exponential
//    multiplied into every term (:865-871).
// libm exp and pow are used as they are: this form is compared with the
// engine within a tolerance, not bit for bit.
int assemble_one_gpu_ref(const AsmCtx& c, int64_t p, double* K, double& eps_out, double& eip_out) {
    const int dim = c.dim;
    const int64_t beg = c.rowptr[p];
    const int k = (int)(c.rowptr[p + 1] - beg);
    const int n = c.B.n;
    std::vector<double> X((size_t)k * dim);
    for (int q = 0; q < k; ++q) {
        const double* xq = c.ps + (size_t)c.cols[beg + q] * dim;
        for (int d = 0; d < dim; ++d) X[(size_t)q * dim + d] = offset1(c.g, d, c.pd[(size_t)p * dim + d], xq[d]);
    }
    for (int q = 0; q < k; ++q) K[q] = 0.0;
    double s = 0.0;
    for (int q = 0; q < k; ++q)
        for (int d = 0; d < dim; ++d) s = s + std::fabs(X[(size_t)q * dim + d]);
    s = s / (double)k;
    const double eps = 2.0 * s;
    eps_out = eps;
    eip_out = 1.0 / std::pow(eps, (double)c.ord);
    if (k < n) return ST_TOO_FEW;
    if (!(eps > 0.0) || !std::isfinite(eps)) return ST_BAD_EPS;
    auto mono_pow = [&](int j, const double* x) {
        double r = (double)c.B.scalars[j];
        for (int d = 0; d < dim; ++d) r = r * std::pow(x[d], (double)c.B.exps[j * dim + d]);
        return r;
    };
    std::vector<double> Bm((size_t)k * n);
    for (int q = 0; q < k; ++q) {
        const double* x = &X[(size_t)q * dim];
        const double e = std::exp(-norm2(dim, x) / (2.0 * eps * eps));
        for (int j = 0; j < n; ++j) {
            unsigned order = 0;
            for (int d = 0; d < dim; ++d) order += c.B.exps[j * dim + d];
            Bm[(size_t)q * n + j] = e * (mono_pow(j, x) / std::pow(eps, (double)order));
        }
    }
    std::vector<double> A((size_t)n * n);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            double acc = 0.0;
            for (int q = 0; q < k; ++q) acc = acc + Bm[(size_t)q * n + i] * Bm[(size_t)q * n + j];
            A[(size_t)i * n + j] = acc;
        }
    // LU without pivoting: A = L U, L unit lower (multipliers below the diagonal)
    for (int col = 0; col < n; ++col) {
        const double piv = A[(size_t)col * n + col];
        if (piv == 0.0 || !std::isfinite(piv)) return ST_SINGULAR;
        for (int r = col + 1; r < n; ++r) {
            const double l = A[(size_t)r * n + col] / piv;
            A[(size_t)r * n + col] = l;
            for (int j = col + 1; j < n; ++j) A[(size_t)r * n + j] = A[(size_t)r * n + j] - l * A[(size_t)col * n + j];
        }
    }
    std::vector<double> a(c.b);
    for (int r = 1; r < n; ++r)
        for (int j = 0; j < r; ++j) a[r] = a[r] - A[(size_t)r * n + j] * a[j];
    for (int r = n - 1; r >= 0; --r) {
        for (int j = r + 1; j < n; ++j) a[r] = a[r] - A[(size_t)r * n + j] * a[j];
        a[r] = a[r] / A[(size_t)r * n + r];
    }
    std::vector<double> u(dim);
    for (int q = 0; q < k; ++q) {
        for (int d = 0; d < dim; ++d) u[d] = X[(size_t)q * dim + d] / eps;
        const double ef = std::exp(-norm2(dim, u.data()));
        double res = 0.0;
        for (int i = 0; i < n; ++i) res = res + a[i] * mono_pow(i, u.data()) * ef;
        K[q] = res;
    }
    for (int q = 0; q < k; ++q)
        if (!std::isfinite(K[q])) {
            for (int r = 0; r < k; ++r) K[r] = 0.0;
            return ST_NONFINITE;
        }
    return ST_OK;
}

}  // namespace

extern "C" {

int orc_version() { return 1; }

double orc_exp(double x) { return cw_exp(x); }

void orc_exp_array(const double* x, double* y, int64_t n) {
    for (int64_t i = 0; i < n; ++i) y[i] = cw_exp(x[i]);
}

double orc_ipow(double x, unsigned e) { return ipow(x, e); }

// Writes the basis of MonomialBasis(sig, order) into exps (n x dim) and
// scalars (n); returns n, or -1 when cap is too small.
int orc_basis(int dim, const unsigned* sig, unsigned order, unsigned* exps, unsigned* scalars, int cap) {
    Basis b = make_basis(dim, sig, order);
    if (b.n > cap) return -1;
    if (exps) std::memcpy(exps, b.exps.data(), sizeof(unsigned) * b.exps.size());
    if (scalars) std::memcpy(scalars, b.scalars.data(), sizeof(unsigned) * b.scalars.size());
    return b.n;
}

int orc_rhs(int dim, const unsigned* sig, unsigned order, double* b, int cap) {
    Basis B = make_basis(dim, sig, order);
    if (B.n > cap) return -1;
    make_rhs(B, sig, b);
    return B.n;
}

void orc_monomial_derivative(int dim, const unsigned* e, unsigned scalar, const unsigned* dord,
                             unsigned* oe, unsigned* os) {
    mono_deriv(dim, e, scalar, dord, oe, os);
}

double orc_monomial_eval(int dim, const unsigned* e, unsigned scalar, const double* x) {
    return mono_eval(dim, e, scalar, x);
}

// Neighbour lists (CSR).  Domain particle p gets every support particle q with
// |x_p - x_q|^2 < rc_p^2 (rc_p = rcut_pp[p] if given, else rcut), skipping
// q == p when self_skip is set; neighbours in ascending q.  Cell list with
// cells no smaller than the largest cutoff.  rowptr has n_dom+1 entries; cols
// may be NULL (count only).  Returns nnz, or -1 if cols_cap is too small.
int64_t orc_neighbors(int dim, const double* pd, int64_t n_dom, const double* ps, int64_t n_sup,
                      int self_skip, double rcut, const double* rcut_pp, const double* box_lo,
                      const double* box_hi, const int* periodic, int64_t* rowptr, int32_t* cols,
                      int64_t cols_cap) {
    double lo[3], hi[3];
    for (int d = 0; d < dim; ++d) {
        if (box_lo && box_hi) {
            lo[d] = box_lo[d];
            hi[d] = box_hi[d];
        } else {
            lo[d] = std::numeric_limits<double>::infinity();
            hi[d] = -lo[d];
            for (int64_t i = 0; i < n_sup; ++i) {
                lo[d] = std::min(lo[d], ps[i * dim + d]);
                hi[d] = std::max(hi[d], ps[i * dim + d]);
            }
            for (int64_t i = 0; i < n_dom; ++i) {
                lo[d] = std::min(lo[d], pd[i * dim + d]);
                hi[d] = std::max(hi[d], pd[i * dim + d]);
            }
        }
    }
    Geom g = make_geom(dim, lo, hi, (box_lo && box_hi) ? periodic : nullptr);
    double rmax = rcut;
    if (rcut_pp)
        for (int64_t i = 0; i < n_dom; ++i) rmax = std::max(rmax, rcut_pp[i]);
    double cmin = rmax * (1.0 + 1e-9);
    int nc[3] = {1, 1, 1};
    double cs[3] = {1, 1, 1};
    for (int d = 0; d < dim; ++d) {
        double Ld = hi[d] - lo[d];
        long m = (cmin > 0) ? (long)std::floor(Ld / cmin) : 1;
        if (m < 1) m = 1;
        if (m > 4096) m = 4096;
        nc[d] = (int)m;
        cs[d] = (Ld > 0) ? Ld / (double)m : 1.0;
    }
    auto cell_of = [&](const double* x, int* c) {
        for (int d = 0; d < dim; ++d) {
            long v = (long)std::floor((x[d] - lo[d]) / cs[d]);
            if (v < 0) v = 0;
            if (v >= nc[d]) v = nc[d] - 1;
            c[d] = (int)v;
        }
    };
    int64_t ncell = (int64_t)nc[0] * nc[1] * nc[2];
    std::vector<int64_t> cstart(ncell + 1, 0);
    std::vector<int32_t> cidx(n_sup);
    std::vector<int64_t> cl(n_sup);
    for (int64_t i = 0; i < n_sup; ++i) {
        int c[3] = {0, 0, 0};
        cell_of(ps + i * dim, c);
        cl[i] = c[0] + (int64_t)nc[0] * (c[1] + (int64_t)nc[1] * c[2]);
        cstart[cl[i] + 1]++;
    }
    for (int64_t c = 0; c < ncell; ++c) cstart[c + 1] += cstart[c];
    {
        std::vector<int64_t> fill(cstart.begin(), cstart.end() - 1);
        for (int64_t i = 0; i < n_sup; ++i) cidx[fill[cl[i]]++] = (int32_t)i;
    }
    rowptr[0] = 0;
    std::vector<int32_t> tmp;
    int64_t nnz = 0;
    for (int64_t p = 0; p < n_dom; ++p) {
        const double* xp = pd + p * dim;
        double rc = rcut_pp ? rcut_pp[p] : rcut;
        double rc2 = rc * rc;
        int c[3] = {0, 0, 0};
        cell_of(xp, c);
        int lst[3][3], cnt[3] = {1, 1, 1};
        for (int d = 0; d < 3; ++d) {
            lst[d][0] = 0;
            if (d >= dim) continue;
            cnt[d] = 0;
            for (int o = -1; o <= 1; ++o) {
                int v = c[d] + o;
                if (g.per[d]) {
                    v = ((v % nc[d]) + nc[d]) % nc[d];
                } else if (v < 0 || v >= nc[d]) {
                    continue;
                }
                bool dup = false;
                for (int t = 0; t < cnt[d]; ++t) dup |= (lst[d][t] == v);
                if (!dup) lst[d][cnt[d]++] = v;
            }
        }
        tmp.clear();
        for (int a2 = 0; a2 < cnt[2]; ++a2)
            for (int a1 = 0; a1 < cnt[1]; ++a1)
                for (int a0 = 0; a0 < cnt[0]; ++a0) {
                    int64_t cc = lst[0][a0] + (int64_t)nc[0] * (lst[1][a1] + (int64_t)nc[1] * lst[2][a2]);
                    for (int64_t t = cstart[cc]; t < cstart[cc + 1]; ++t) {
                        int32_t q = cidx[t];
                        if (self_skip && q == p) continue;
                        double o[3];
                        for (int d = 0; d < dim; ++d) o[d] = offset1(g, d, xp[d], ps[(int64_t)q * dim + d]);
                        if (norm2(dim, o) < rc2) tmp.push_back(q);
                    }
                }
        std::sort(tmp.begin(), tmp.end());
        if (cols) {
            if (nnz + (int64_t)tmp.size() > cols_cap) return -1;
            std::copy(tmp.begin(), tmp.end(), cols + nnz);
        }
        nnz += (int64_t)tmp.size();
        rowptr[p + 1] = nnz;
    }
    return nnz;
}

// Same predicate by exhaustive search (for checking the cell version).
int64_t orc_neighbors_brute(int dim, const double* pd, int64_t n_dom, const double* ps, int64_t n_sup,
                            int self_skip, double rcut, const double* rcut_pp, const double* box_lo,
                            const double* box_hi, const int* periodic, int64_t* rowptr, int32_t* cols,
                            int64_t cols_cap) {
    Geom g = make_geom(dim, box_lo, box_hi, periodic);
    int64_t nnz = 0;
    rowptr[0] = 0;
    for (int64_t p = 0; p < n_dom; ++p) {
        double rc = rcut_pp ? rcut_pp[p] : rcut;
        double rc2 = rc * rc;
        for (int64_t q = 0; q < n_sup; ++q) {
            if (self_skip && q == p) continue;
            double o[3];
            for (int d = 0; d < dim; ++d) o[d] = offset1(g, d, pd[p * dim + d], ps[q * dim + d]);
            if (norm2(dim, o) < rc2) {
                if (cols) {
                    if (nnz >= cols_cap) return -1;
                    cols[nnz] = (int32_t)q;
                }
                ++nnz;
            }
        }
        rowptr[p + 1] = nnz;
    }
    return nnz;
}

// One reference Dcpse object: eps, epsInvPow and the kernels (calcKernels in
// neighbour order) for every domain particle.  status[p] != 0 marks a particle
// whose system could not be built (kernels set to zero).  Returns the number
// of such particles.
int64_t orc_assemble_mode(int dim, const double* pd, int64_t n_dom, const double* ps, const int64_t* rowptr,
                          const int32_t* cols, const double* box_lo, const double* box_hi, const int* periodic,
                          const unsigned* sig, unsigned order, double h_over_eps, const double* eps_fixed,
                          double* eps, double* eps_inv_pow, double* kernels, int32_t* status, int nthreads,
                          int exact_gram) {
    AsmCtx c;
    c.exact_gram = exact_gram != 0;
    c.dim = dim;
    c.pd = pd;
    c.ps = ps;
    c.rowptr = rowptr;
    c.cols = cols;
    c.g = make_geom(dim, box_lo, box_hi, periodic);
    c.B = make_basis(dim, sig, order);
    c.b.resize(c.B.n);
    make_rhs(c.B, sig, c.b.data());
    c.ord = 0;
    for (int d = 0; d < dim; ++d) c.ord += sig[d];
    c.hoe = h_over_eps;
    c.eps_fixed = eps_fixed;
    std::vector<int64_t> bad(std::max(nthreads, 1), 0);
    parallel_for(n_dom, nthreads, [&](int64_t b, int64_t e) {
        int64_t nb = 0;
        for (int64_t p = b; p < e; ++p) {
            double ep, eip;
            int st = assemble_one(c, p, kernels + rowptr[p], ep, eip);
            eps[p] = ep;
            eps_inv_pow[p] = eip;
            status[p] = st;
            nb += (st != 0);
        }
        // accumulate without a lock: one slot per range start
        __atomic_fetch_add(&bad[0], nb, __ATOMIC_RELAXED);
    });
    return bad[0];
}

int64_t orc_assemble(int dim, const double* pd, int64_t n_dom, const double* ps, const int64_t* rowptr,
                     const int32_t* cols, const double* box_lo, const double* box_hi, const int* periodic,
                     const unsigned* sig, unsigned order, double h_over_eps, const double* eps_fixed,
                     double* eps, double* eps_inv_pow, double* kernels, int32_t* status, int nthreads) {
    return orc_assemble_mode(dim, pd, n_dom, ps, rowptr, cols, box_lo, box_hi, periodic, sig, order, h_over_eps,
                             eps_fixed, eps, eps_inv_pow, kernels, status, nthreads, 0);
}

// Dcpse_gpu's assembly (Dcpse.cuh:776-875) of one reference Dcpse_gpu object
// over the given lists; same arguments and outputs as orc_assemble, without
// h_over_eps and eps_fixed (the GPU class has neither).
int64_t orc_assemble_gpu_ref(int dim, const double* pd, int64_t n_dom, const double* ps, const int64_t* rowptr,
                             const int32_t* cols, const double* box_lo, const double* box_hi, const int* periodic,
                             const unsigned* sig, unsigned order, double* eps, double* eps_inv_pow, double* kernels,
                             int32_t* status, int nthreads) {
    AsmCtx c;
    c.dim = dim;
    c.pd = pd;
    c.ps = ps;
    c.rowptr = rowptr;
    c.cols = cols;
    c.g = make_geom(dim, box_lo, box_hi, periodic);
    c.B = make_basis(dim, sig, order);
    c.b.resize(c.B.n);
    make_rhs(c.B, sig, c.b.data());
    c.ord = 0;
    for (int d = 0; d < dim; ++d) c.ord += sig[d];
    c.hoe = 0.5;
    c.eps_fixed = nullptr;
    std::vector<int64_t> bad(1, 0);
    parallel_for(n_dom, nthreads, [&](int64_t b, int64_t e) {
        int64_t nb = 0;
        for (int64_t p = b; p < e; ++p) {
            double ep, eip;
            int st = assemble_one_gpu_ref(c, p, kernels + rowptr[p], ep, eip);
            eps[p] = ep;
            eps_inv_pow[p] = eip;
            status[p] = st;
            nb += (st != 0);
        }
        __atomic_fetch_add(&bad[0], nb, __ATOMIC_RELAXED);
    });
    return bad[0];
}

// Dcpse.hpp:467-499: Df_p = epsInvPow_p * sum_q (f_q + sign f_p) K_pq,
// sign = -1 for even |alpha|.
void orc_apply(int64_t n_dom, const double* f_sup, const double* f_dom, const int64_t* rowptr,
               const int32_t* cols, const double* kernels, const double* eps_inv_pow, unsigned diff_order,
               double* out, int nthreads) {
    const double sign = (diff_order % 2 == 0) ? -1.0 : 1.0;
    parallel_for(n_dom, nthreads, [&](int64_t b, int64_t e) {
        for (int64_t p = b; p < e; ++p) {
            double fxp = sign * f_dom[p];
            double D = 0.0;
            for (int64_t j = rowptr[p]; j < rowptr[p + 1]; ++j) D = D + (f_sup[cols[j]] + fxp) * kernels[j];
            out[p] = D * eps_inv_pow[p];
        }
    });
}

// VECT_DCPSE_V_SUM (DCPSE_op.hpp:388-399): out_p = sum_c D_c f (p), in
// component order, for `ncomp` reference Dcpse objects sharing the list.
void orc_apply_sum(int64_t n_dom, int ncomp, const double* f_sup, const double* f_dom, const int64_t* rowptr,
                   const int32_t* cols, const double* const* kernels, const double* const* eps_inv_pow,
                   const unsigned* diff_order, double* out, int nthreads) {
    parallel_for(n_dom, nthreads, [&](int64_t b, int64_t e) {
        for (int64_t p = b; p < e; ++p) {
            double v = 0.0;
            for (int c = 0; c < ncomp; ++c) {
                const double sign = (diff_order[c] % 2 == 0) ? -1.0 : 1.0;
                double fxp = sign * f_dom[p];
                double D = 0.0;
                for (int64_t j = rowptr[p]; j < rowptr[p + 1]; ++j)
                    D = D + (f_sup[cols[j]] + fxp) * kernels[c][j];
                v = v + D * eps_inv_pow[c][p];
            }
            out[p] = v;
        }
    });
}

// Reference adjoint (FP64) of y_o,p = sum_q W_o,pq (f_q - f_p) with respect
// to positions, W_o = sum_{t in o} eps_p^-|alpha_t| K_t (the weights of
// Dcpse.hpp:690-809), neighbour lists fixed.  Written per term directly from
// K_t,q = omega_q v_q^T a_t, a_t = A^-1 b_t, A = sum_q omega_q v_q v_q^T,
// omega_q = exp(-|u_q|^2), u_q = x_pq / eps,
// eps = sum_q |x_pq|_1 / (k HOverEpsilon):
//   Phi_t = g_o(t),p e_t s^T a_t,  s = sum_q c_q omega_q v_q, lambda = A^-1 s,
//   dPhi/domega_q = e g (v.a)(c - v.lambda), dPhi/dv_q = e g omega ((c - v.lambda) a - (v.a) lambda),
// then the chain rule through u_q, eps and e_t = eps^-|alpha_t|.
// grad is [n][dim] and accumulated (zero it first).  Positions, f, g: domain
// arrays; sigs: nterms x dim; term_output: output of each term; g: [nout][n].
}  // extern "C"

namespace {
// The adjoint of rows [row0, row1): emit(i, d, v) adds v to d/dx_i,d.
template <typename Emit>
int64_t vjp_rows(int dim, const double* pos, int64_t n, const int64_t* rowptr, const int32_t* cols, int nterms,
                 const unsigned* sigs, const int* term_output, unsigned order, double h_over_eps, const double* f,
                 const double* g, int64_t row0, int64_t row1, Emit emit) {
    Geom geo = make_geom(dim, nullptr, nullptr, nullptr);
    std::vector<Basis> bases;
    std::vector<std::vector<double>> rhs;
    for (int t = 0; t < nterms; ++t) {
        bases.push_back(make_basis(dim, sigs + t * dim, order));
        std::vector<double> b(bases.back().n);
        make_rhs(bases.back(), sigs + t * dim, b.data());
        rhs.push_back(b);
    }
    int64_t skipped = 0;
    for (int64_t p = row0; p < row1; ++p) {
        const int64_t beg = rowptr[p];
        const int k = (int)(rowptr[p + 1] - beg);
        std::vector<double> X((size_t)k * dim);
        double s1 = 0.0;
        for (int q = 0; q < k; ++q)
            for (int d = 0; d < dim; ++d) {
                X[(size_t)q * dim + d] = offset1(geo, d, pos[p * dim + d], pos[(int64_t)cols[beg + q] * dim + d]);
                s1 += std::fabs(X[(size_t)q * dim + d]);
            }
        const double eps = s1 / k / h_over_eps;
        bool ok = k > 0 && eps > 0 && std::isfinite(eps);
        for (int t = 0; t < nterms && ok; ++t) ok = k >= bases[t].n;
        if (!ok) {
            ++skipped;
            continue;
        }
        std::vector<double> U((size_t)k * dim), om(k), c(k);
        for (int q = 0; q < k; ++q) {
            double r2 = 0.0;
            for (int d = 0; d < dim; ++d) {
                U[(size_t)q * dim + d] = X[(size_t)q * dim + d] / eps;
                r2 += U[(size_t)q * dim + d] * U[(size_t)q * dim + d];
            }
            om[q] = std::exp(-r2);
            c[q] = f[cols[beg + q]] - f[p];
        }
        std::vector<double> Gq((size_t)k * dim, 0.0);  // dPhi / du_q
        double dPhi_deps_explicit = 0.0;
        for (int t = 0; t < nterms; ++t) {
            const Basis& B = bases[t];
            const int nb = B.n;
            const double gt = g[(int64_t)term_output[t] * n + p];
            unsigned m = 0;
            for (int d = 0; d < dim; ++d) m += sigs[t * dim + d];
            const double et = 1.0 / std::pow(eps, (double)m);
            std::vector<double> V((size_t)k * nb), dV((size_t)k * nb * dim);
            for (int q = 0; q < k; ++q)
                for (int i = 0; i < nb; ++i) {
                    const unsigned* e = &B.exps[i * dim];
                    double val = 1.0;
                    for (int d = 0; d < dim; ++d) val *= std::pow(U[(size_t)q * dim + d], (double)e[d]);
                    V[(size_t)q * nb + i] = val;
                    for (int d = 0; d < dim; ++d) {
                        double dv = 0.0;
                        if (e[d] > 0) {
                            dv = e[d] * std::pow(U[(size_t)q * dim + d], (double)e[d] - 1.0);
                            for (int d2 = 0; d2 < dim; ++d2)
                                if (d2 != d) dv *= std::pow(U[(size_t)q * dim + d2], (double)e[d2]);
                        }
                        dV[((size_t)q * nb + i) * dim + d] = dv;
                    }
                }
            std::vector<double> A((size_t)nb * nb, 0.0), sv(nb, 0.0);
            for (int q = 0; q < k; ++q)
                for (int i = 0; i < nb; ++i) {
                    sv[i] += c[q] * om[q] * V[(size_t)q * nb + i];
                    for (int j = 0; j < nb; ++j) A[(size_t)i * nb + j] += om[q] * V[(size_t)q * nb + i] * V[(size_t)q * nb + j];
                }
            std::vector<double> C(2 * (size_t)nb), sol(2 * (size_t)nb);
            for (int i = 0; i < nb; ++i) {
                C[i * 2] = rhs[t][i];
                C[i * 2 + 1] = sv[i];
            }
            std::vector<double> Ac(A);
            if (!cpqr_solve(nb, 2, Ac.data(), C.data(), sol.data())) {
                ok = false;
                break;
            }
            double sa = 0.0;
            for (int i = 0; i < nb; ++i) sa += sv[i] * sol[i * 2];
            dPhi_deps_explicit += gt * (-(double)m) * et * sa / eps;
            for (int q = 0; q < k; ++q) {
                double va = 0.0, vl = 0.0;
                for (int i = 0; i < nb; ++i) {
                    va += V[(size_t)q * nb + i] * sol[i * 2];
                    vl += V[(size_t)q * nb + i] * sol[i * 2 + 1];
                }
                const double dom = gt * et * va * (c[q] - vl);
                for (int d = 0; d < dim; ++d) {
                    double acc = dom * (-2.0 * om[q] * U[(size_t)q * dim + d]);
                    for (int i = 0; i < nb; ++i) {
                        const double beta = gt * et * om[q] * ((c[q] - vl) * sol[i * 2] - va * sol[i * 2 + 1]);
                        acc += beta * dV[((size_t)q * nb + i) * dim + d];
                    }
                    Gq[(size_t)q * dim + d] += acc;
                }
            }
        }
        if (!ok) {
            ++skipped;
            continue;
        }
        double gu_dot_u = 0.0;
        for (int q = 0; q < k; ++q)
            for (int d = 0; d < dim; ++d) gu_dot_u += Gq[(size_t)q * dim + d] * U[(size_t)q * dim + d];
        const double Dtot = dPhi_deps_explicit - gu_dot_u / eps;
        for (int q = 0; q < k; ++q) {
            const int64_t qq = cols[beg + q];
            for (int d = 0; d < dim; ++d) {
                const double x = X[(size_t)q * dim + d];
                const double sg = x > 0 ? 1.0 : (x < 0 ? -1.0 : 0.0);
                const double G = Gq[(size_t)q * dim + d] / eps + Dtot * sg / (k * h_over_eps);
                emit(p, d, G);
                emit(qq, d, -G);
            }
        }
    }
    return skipped;
}
}  // namespace

extern "C" {

int64_t orc_vjp_positions(int dim, const double* pos, int64_t n, const int64_t* rowptr, const int32_t* cols,
                          int nterms, const unsigned* sigs, const int* term_output, unsigned order, double h_over_eps,
                          const double* f, const double* g, double* grad) {
    return vjp_rows(dim, pos, n, rowptr, cols, nterms, sigs, term_output, order, h_over_eps, f, g, 0, n,
                    [&](int64_t i, int d, double v) { grad[i * dim + d] += v; });
}

// The same for rows [row0, row1) on nthreads threads: each thread records
// its contributions, which are then added in thread order (grad is not
// zeroed first).
int64_t orc_vjp_positions_rows(int dim, const double* pos, int64_t n, const int64_t* rowptr, const int32_t* cols,
                               int nterms, const unsigned* sigs, const int* term_output, unsigned order,
                               double h_over_eps, const double* f, const double* g, int64_t row0, int64_t row1,
                               int nthreads, double* grad) {
    const int nt = std::max(1, nthreads);
    struct Part {
        std::vector<int64_t> idx;
        std::vector<double> val;
        int64_t skipped = 0;
    };
    std::vector<Part> parts((size_t)nt);
    const int64_t rows = row1 - row0;
    const int64_t chunk = (rows + nt - 1) / nt;
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t) {
        const int64_t b = row0 + t * chunk, e = std::min(row1, b + chunk);
        if (b >= e) continue;
        th.emplace_back([&, t, b, e] {
            Part& P = parts[(size_t)t];
            P.skipped = vjp_rows(dim, pos, n, rowptr, cols, nterms, sigs, term_output, order, h_over_eps, f, g, b, e,
                                 [&](int64_t i, int d, double v) {
                                     P.idx.push_back(i * dim + d);
                                     P.val.push_back(v);
                                 });
        });
    }
    for (auto& x : th) x.join();
    int64_t skipped = 0;
    for (auto& P : parts) {
        for (size_t j = 0; j < P.idx.size(); ++j) grad[P.idx[j]] += P.val[j];
        skipped += P.skipped;
    }
    return skipped;
}

// Several outputs in one sweep over the particles, the way the reference's
// expression evaluation visits them (vector_dist_op_compute_op<prp,comp_host>
// ::compute_expr, src/Operators/Vector/cuda/vector_dist_operators_cuda.cuh:
// 447-461): for each particle, each output, its terms in order
// (VECT_DCPSE_V_SUM / VECT_DCPSE_V, DCPSE_op.hpp:144-153, 388-399).
// term_output[t] gives the output of term t; out is [nout][n_dom].
void orc_apply_multi(int64_t n_dom, int nterms, const double* f_sup, const double* f_dom, const int64_t* rowptr,
                     const int32_t* cols, const double* const* kernels, const double* const* eps_inv_pow,
                     const unsigned* diff_order, const int* term_output, int nout, double* out, int nthreads) {
    parallel_for(n_dom, nthreads, [&](int64_t b, int64_t e) {
        for (int64_t p = b; p < e; ++p) {
            for (int o = 0; o < nout; ++o) {
                double v = 0.0;
                for (int c = 0; c < nterms; ++c) {
                    if (term_output[c] != o) continue;
                    const double sign = (diff_order[c] % 2 == 0) ? -1.0 : 1.0;
                    double fxp = sign * f_dom[p];
                    double D = 0.0;
                    for (int64_t j = rowptr[p]; j < rowptr[p + 1]; ++j) D = D + (f_sup[cols[j]] + fxp) * kernels[c][j];
                    v = v + D * eps_inv_pow[c][p];
                }
                out[(int64_t)o * n_dom + p] = v;
            }
        }
    });
}

// Dcpse::p2p (Dcpse.hpp:198-227 scalar, :239-297 vector of N1 components):
// Df_p = epsInvPow_p * sum_q f_q K_pq with f on the support set and no f_p
// term; the components are independent sums in neighbour order.
void orc_p2p(int64_t n_dom, int ncomp, const double* f_sup, const int64_t* rowptr, const int32_t* cols,
             const double* kernels, const double* eps_inv_pow, double* out, int nthreads) {
    parallel_for(n_dom, nthreads, [&](int64_t b, int64_t e) {
        std::vector<double> D((size_t)ncomp);
        for (int64_t p = b; p < e; ++p) {
            for (int c = 0; c < ncomp; ++c) D[c] = 0.0;
            for (int64_t j = rowptr[p]; j < rowptr[p + 1]; ++j)
                for (int c = 0; c < ncomp; ++c) D[c] = D[c] + f_sup[(int64_t)cols[j] * ncomp + c] * kernels[j];
            for (int c = 0; c < ncomp; ++c) out[p * ncomp + c] = eps_inv_pow[p] * D[c];
        }
    });
}

// Operator matrix rows as DCPSE_scheme::impose_git (DCPSE_Solver.hpp:980-1030)
// collects them from value_nz (DCPSE_op.hpp:70-83 one Dcpse, :405-420 a sum
// of Dcpse objects): per row a map column -> coefficient, filled by
//   for term t, neighbour j:  cols[q_j] += (K_tj * coeff) * eip_t(p);
//                             cols[p]   += ((sign_t * K_tj) * coeff) * eip_t(p)
// then a zero diagonal if none was set; written out in ascending columns.
// Two calls: out_cols == NULL fills out_rowptr only.
void orc_operator_csr(int64_t nrows, const int64_t* rows, const int64_t* rowptr, const int32_t* cols, int nterms,
                      const double* const* K, const double* const* eip, const double* sign, double coeff,
                      int64_t nvar, int64_t var, int64_t* out_rowptr, int64_t* out_cols, double* out_vals) {
    out_rowptr[0] = 0;
    for (int64_t r = 0; r < nrows; ++r) {
        const int64_t p = rows ? rows[r] : r;
        std::map<int64_t, double> m;
        for (int t = 0; t < nterms; ++t)
            for (int64_t j = rowptr[p]; j < rowptr[p + 1]; ++j) {
                const double kc = K[t][j] * coeff;
                m[(int64_t)cols[j] * nvar + var] += kc * eip[t][p];
                const double skc = (sign[t] * K[t][j]) * coeff;
                m[p * nvar + var] += skc * eip[t][p];
            }
        if (m.find(p * nvar + var) == m.end()) m[p * nvar + var] = 0.0;
        int64_t o = out_rowptr[r];
        if (out_cols)
            for (const auto& kv : m) {
                out_cols[o] = kv.first;
                out_vals[o] = kv.second;
                ++o;
            }
        out_rowptr[r + 1] = out_rowptr[r] + (int64_t)m.size();
    }
}

// SurfaceDcpse::createNormalParticles (Dcpse.hpp:855-876): after the nb base
// (surface) particles come 2*n_count virtual particles per base particle p,
// for i = 1..n_count first x_p + i*s_p*n_p then x_p - i*s_p*n_p, each
// coordinate xp[j] + (i*s_p)*N[j] (resp. minus), with s_p = spacings[p] if
// given (support_options::ADAPTIVE), else spacing.  out holds
// nb*(1 + 2*n_count) positions.
void orc_surface_extend(int dim, const double* base, const double* normals, int64_t nb, int n_count, double spacing,
                        const double* spacings, double* out) {
    for (int64_t p = 0; p < nb * dim; ++p) out[p] = base[p];
    int64_t v = nb;
    for (int64_t p = 0; p < nb; ++p) {
        const double s = spacings ? spacings[p] : spacing;
        for (int i = 1; i <= n_count; ++i) {
            const double is = (double)i * s;
            for (int j = 0; j < dim; ++j) out[v * dim + j] = base[p * dim + j] + is * normals[p * dim + j];
            ++v;
            for (int j = 0; j < dim; ++j) out[v * dim + j] = base[p * dim + j] - is * normals[p * dim + j];
            ++v;
        }
    }
}

// SurfaceDcpse::accumulateAndDeleteNormalParticles (Dcpse.hpp:947-1015): the
// kernels of every virtual support particle are added onto its base particle
// (q < nb: itself; else (q - nb) / (2 n_count)); the new list holds each base
// particle once, in order of first appearance, with the running sums
// (first value, then += in list order).  Two calls: out_cols == NULL fills
// out_rowptr only.  nterms kernel arrays share the list.
void orc_surface_accumulate(int64_t n_dom, int64_t nb, int n_count, const int64_t* rowptr, const int32_t* cols,
                            int nterms, const double* const* K, int64_t* out_rowptr, int32_t* out_cols,
                            double* const* out_K) {
    out_rowptr[0] = 0;
    std::vector<int64_t> seen;
    for (int64_t p = 0; p < n_dom; ++p) {
        seen.clear();
        const int64_t o = out_rowptr[p];
        for (int64_t j = rowptr[p]; j < rowptr[p + 1]; ++j) {
            const int64_t q = cols[j];
            const int64_t real = (q < nb) ? q : (q - nb) / (2 * (int64_t)n_count);
            int64_t slot = -1;
            for (size_t s2 = 0; s2 < seen.size(); ++s2)
                if (seen[s2] == real) slot = (int64_t)s2;
            if (slot < 0) {
                slot = (int64_t)seen.size();
                seen.push_back(real);
                if (out_cols) {
                    out_cols[o + slot] = (int32_t)real;
                    for (int t = 0; t < nterms; ++t) out_K[t][o + slot] = K[t][j];
                }
            } else if (out_cols) {
                for (int t = 0; t < nterms; ++t) out_K[t][o + slot] = out_K[t][o + slot] + K[t][j];
            }
        }
        out_rowptr[p + 1] = o + (int64_t)seen.size();
    }
}

}  // extern "C"
