// dcpse_matrix.cu -- operator matrices in CSR form for implicit solves.
//
// Replaces the row construction of DCPSE_scheme::impose_git
// (src/DCPSE/DCPSE_op/DCPSE_Solver.hpp:980-1030), which asks every operator
// node for its non-zeros through value_nz (src/DCPSE/DCPSE_op/DCPSE_op.hpp:
// 70-83 for one Dcpse, :405-420 for a sum of Dcpse objects such as the
// Laplacian) and collects them in a hash map per row:
//     for each term i of the output, for each neighbour j of p:
//         cols[q_j] += (K_ij * coeff) * eip_i(p)
//         cols[p]   += ((sign_i * K_ij) * coeff) * eip_i(p)
// with sign_i = Dcpse::getSign() (-1 for even nonzero |alpha|, else +1,
// Dcpse.hpp:533-541).  Here one thread builds one row with the same
// additions in the same order: every off-diagonal entry sums its terms in
// term order, the diagonal sums over terms and neighbours in visiting order
// (including the neighbour's own entry when p is in its list).  Columns come
// out ascending with the diagonal at its place; a row without neighbours
// holds a zero diagonal, as impose_git adds one.
#include "dcpse_internal.h"

namespace dcpse {
namespace {

__device__ __forceinline__ int64_t row_particle(const int64_t* rows, int64_t r) { return rows ? rows[r] : r; }

__global__ void csr_count_kernel(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ cols,
                                 const int64_t* __restrict__ rows, int64_t nrows, int32_t* __restrict__ counts) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nrows; r += (int64_t)gridDim.x * blockDim.x) {
        const int64_t p = row_particle(rows, r);
        const int64_t b = rowptr[p], e = rowptr[p + 1];
        bool self = false;
        for (int64_t j = b; j < e; ++j) self |= (cols[j] == (int32_t)p);
        counts[r] = (int32_t)(e - b) + (self ? 0 : 1);
    }
}

__global__ void csr_fill_kernel(MatArgs a) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < a.nrows; r += (int64_t)gridDim.x * blockDim.x) {
        const int64_t p = row_particle(a.rows, r);
        const int64_t b = a.rowptr[p], e = a.rowptr[p + 1];
        // diagonal in visiting order: terms, then neighbours
        double diag = 0.0;
        for (int t = 0; t < a.nterms; ++t) {
            const double* K = a.K[t];
            const double eip = a.eip[t][p];
            for (int64_t j = b; j < e; ++j) {
                if (a.cols[j] == (int32_t)p) diag = diag + (K[j] * a.coeff) * eip;
                diag = diag + ((a.sign[t] * K[j]) * a.coeff) * eip;
            }
        }
        int64_t o = a.out_rowptr[r];
        bool placed = false;
        for (int64_t j = b; j < e; ++j) {
            const int64_t q = a.cols[j];
            if (!placed && q >= p) {
                a.out_cols[o] = p * a.nvar + a.var;
                a.out_vals[o] = diag;
                ++o;
                placed = true;
                if (q == p) continue;  // its contributions are in the diagonal
            }
            double v = 0.0;
            for (int t = 0; t < a.nterms; ++t) v = v + (a.K[t][j] * a.coeff) * a.eip[t][p];
            a.out_cols[o] = q * a.nvar + a.var;
            a.out_vals[o] = v;
            ++o;
        }
        if (!placed) {
            a.out_cols[o] = p * a.nvar + a.var;
            a.out_vals[o] = diag;
        }
    }
}

int grid_for_rows(int64_t n) {
    int64_t g = (n + 255) / 256;
    const int64_t cap = (int64_t)num_sms() * 8;
    return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

}  // namespace

cudaError_t csr_row_counts(const int64_t* rowptr, const int32_t* cols, const int64_t* rows, int64_t nrows,
                           int32_t* counts, cudaStream_t s) {
    if (nrows == 0) return cudaSuccess;
    csr_count_kernel<<<grid_for_rows(nrows), 256, 0, s>>>(rowptr, cols, rows, nrows, counts);
    return cudaGetLastError();
}

cudaError_t csr_fill(const MatArgs& a, cudaStream_t s) {
    if (a.nrows == 0) return cudaSuccess;
    csr_fill_kernel<<<grid_for_rows(a.nrows), 256, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace dcpse
