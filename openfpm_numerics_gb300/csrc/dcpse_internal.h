// dcpse_internal.h -- host-side interfaces between the C-ABI layer and the
// kernel translation units of the GB300 DC-PSE path.
#pragma once

#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "dcpse_common.cuh"
#include "openfpm_dcpse/dcpse_capi.h"

#define DCPSE_ASSEMBLE_FAST_FLAG DCPSE_ASSEMBLE_FAST

namespace dcpse {

// ------------------------------------------------------------ neighbours --
struct CellGrid {
    double lo[kMaxDim];
    double cs[kMaxDim];
    int nc[kMaxDim];
};

// Exclusive scan of n int32 counts into out[0..n] (out[n] = total).
// tmp must hold scan_tmp_elems(n) int64 values.
int64_t scan_tmp_elems(int64_t n);
cudaError_t exclusive_scan_i32(const int32_t* in, int64_t n, int64_t* out, int64_t* tmp, cudaStream_t s);

// Bounding box of n_a + n_b points (lo/hi written to host arrays).
cudaError_t bounding_box(int dim, const double* a, int64_t na, const double* b, int64_t nb, double* lo,
                         double* hi, unsigned long long* d_tmp /* 2*kMaxDim */, cudaStream_t s);

// Cell list of the support set: cell_start[ncell+1], cidx[n], spos[n*dim]
// (positions in cell order) and srel[n] (FP32 offsets from the cell's lower
// corner, NaN for particles outside the grid).  d_cell (n) and d_fill
// (ncell) are scratch.
// Particles in a renumbering order for the apply's layout: mode 0, the
// Z-order (Morton order) of their cells (cell coordinates coarsened so that
// a key has at most kOrderKeyBits bits), whose windows of consecutive rows
// cover compact blocks of cells; mode 1, row-major order of a grid at the
// particles' mean spacing (close to a jittered lattice's own order).
// tmp: order_tmp_elems() int64; key: n int32.
constexpr int kOrderKeyBits = 23;
int64_t order_tmp_elems(int dim, int64_t n, const CellGrid& g, int mode);
cudaError_t particle_order(int dim, const double* pos, int64_t n, const CellGrid& g, int mode, int32_t* key,
                           int64_t* tmp, int32_t* order, cudaStream_t s);
cudaError_t build_cells(int dim, const double* pos, int64_t n, const CellGrid& g, int32_t* d_cell,
                        int32_t* d_ccount, int64_t* d_cstart, int64_t* d_fill, int32_t* d_cidx, double* d_spos,
                        float4* d_srel, int64_t* d_scan_tmp, cudaStream_t s);

struct NbrArgs {
    int dim;
    const double* pd;   // domain positions
    int64_t n_dom;
    const double* spos; // support positions, cell order
    const float4* srel; // the same, FP32 offsets from the cell's lower corner
    const int32_t* cidx;
    const int64_t* cstart;
    CellGrid cells;
    Geom geom;
    double rcut;
    const double* rcut_pp;
    int self_skip;
    double band;        // |d^2 - rc^2| below this: decided in FP64
    int fast;           // 0: FP64 for every candidate
    float csf[3];       // cell sides in FP32
    int packed;         // cells >= rc / 2, +-2 stencil, packed candidate rows
};

// Count pass: counts[p] = number of neighbours; also atomically maxes *d_maxk.
cudaError_t count_neighbors(const NbrArgs& a, int32_t* counts, int* d_maxk, cudaStream_t s);
// Fill pass: unsorted neighbours of p into tmp[rowptr[p] ...], then sorted
// ascending into cols (maxk: the longest row, from the count pass).
cudaError_t fill_neighbors(const NbrArgs& a, const int64_t* rowptr, int32_t* tmp, int32_t* cols, int maxk,
                           cudaStream_t s);

// --------------------------------------------------------------- assembly --
// Tables describing the bases of a plan, resident on the device.
constexpr int kMaxUnion = 128;   // distinct monomials over all bases
constexpr int kMaxGroups = 4;    // distinct |alpha| among the terms
constexpr int kMaxBasis = 120;   // basis size per group (3D |alpha| = 6, order 2: Laplace_Beltrami)
constexpr int kMaxBasisSmall = 35;  // kernels with per-thread basis arrays (3D order 4 = 34)
constexpr int kMaxTerms = 16;    // reference Dcpse objects per plan
constexpr int kMaxOutputs = 8;
constexpr int kMaxRhs = 8;       // right-hand sides per group
constexpr int kMaxPairs = 8256;  // Gram entries (i <= j) needed by some group (128 x 129 / 2)
constexpr int kMaxExp = 8;       // highest exponent + 1
constexpr int kMaxSlots = 255;   // monomial program: inputs, constant and products (byte indices)

struct AsmTables {
    int dim;
    int nu;                       // union basis size
    unsigned char uexp[kMaxUnion][kMaxDim];
    int maxexp;                   // largest exponent over the union, plus one
    int npairs;
    unsigned char pi[kMaxPairs], pj[kMaxPairs];  // union indices, pi <= pj
    short upair[kMaxUnion][kMaxUnion];           // (lo, hi) union indices -> pair
    int ngroups;
    int gn[kMaxGroups];           // basis size
    int gord[kMaxGroups];         // |alpha| of the group
    unsigned char gidx[kMaxGroups][kMaxBasis];   // group basis -> union index
    // right-hand sides per group: columns either per term (faithful mode) or
    // per output (fast mode)
    int nterm_rhs[kMaxGroups];
    int term_of_rhs[kMaxGroups][kMaxRhs];        // term id of each faithful rhs
    int nout_rhs[kMaxGroups];
    int out_of_rhs[kMaxGroups][kMaxRhs];         // output id of each fast rhs
    double b_term[kMaxGroups][kMaxRhs][kMaxBasis];
    double b_out[kMaxGroups][kMaxRhs][kMaxBasis];
    int nterms;
    int term_group[kMaxTerms];
    int term_output[kMaxTerms];
    int noutputs;
    // Monomial program: per-lane value slots [0, dim) hold u, slot dim holds
    // 1.0, and step s writes slot dim + 1 + s = slot prog[s][0] * slot
    // prog[s][1].  The steps are exactly the multiplications of ipow and of
    // the left-to-right monomial product, each shared value computed once
    // (factors equal to 1.0 are skipped: x * 1.0 == x).
    int nprog;
    int nslots;
    unsigned char prog[kMaxSlots][2];
    unsigned char uslot[kMaxUnion];              // slot holding union monomial j
};

struct AsmArgs {
    const AsmTables* tab;  // device copy
    int dim;
    int64_t n;
    const double* pos;     // domain positions (the rows)
    const double* spos;    // support positions (the columns); pos for one set
    const int64_t* rowptr;
    const int32_t* cols;
    Geom geom;
    double h_over_eps;
    const double* eps_fixed;
    int flags;
    // outputs
    double* eps;
    int32_t* status;
    double* eip_group;   // [ngroups][n]
    double* k_term;      // [nterms][nnz]   (faithful kernels) or nullptr
    double* w64;         // [noutputs][nnz] (summed, eps folded) or nullptr
    float* w32;          // [noutputs][nnz] or nullptr
    void* r16;           // bf16 [noutputs][nnz]: w64 - w32, or nullptr
    float* r32;          // FP32 [noutputs][nnz]: w64 - w32, or nullptr
    int64_t nnz;
    const int32_t* order; // processing order of the particles (k-binned) or nullptr
    int warps;            // warps per CTA of the Gram and weight kernels (2, 4 or 8)
    int qr_lanes;         // lanes per particle of the QR kernel (0 = automatic)
    int maxk;             // longest neighbour row
    double* scratch;      // assembly_scratch_bytes() per particle of a batch
    int64_t scratch_particles;  // batch size the scratch holds
    int* err;             // device error word (bounded waits of the tensor-core Gram)
    double* qws;          // global QR work space for bases too large for shared memory, or nullptr
};

// Scratch bytes per particle of an assembly batch (Gram entries,
// coefficients, the scaled offsets of its rows and a status word) for the
// plan's tables and flags and the longest row maxk.
int64_t assembly_scratch_bytes(const AsmTables& h, int flags, int maxk);
// bytes of the global QR work space an assembly with these tables and flags
// needs (0 when the QR's work space fits in shared memory)
int64_t assembly_qr_ws_bytes(const AsmTables& h, int flags);

// Particle order binned by neighbour count: bins of `width` counts
// ascending (a counting sort on k / width); order[n], tmp sized by
// binning_tmp_elems.
int64_t binning_tmp_elems(int64_t n, int maxk, int width);
cudaError_t bin_by_count(const int64_t* rowptr, int64_t n, int maxk, int width, int32_t* order, int32_t* tmp32,
                         int64_t* tmp64, cudaStream_t s);

// h: host copy of *a.tab (launch configuration is derived from it)
cudaError_t assemble(const AsmArgs& a, const AsmTables& h, cudaStream_t s);
// whether an assembly with these tables, flags and longest row takes its
// Gram products on the tensor cores (DCPSE_ASSEMBLE_TC with the fast
// assembly, at most 32 union monomials and 128 neighbours)
bool assembly_uses_tc(const AsmTables& h, int flags, int maxk);


// ----------------------------------------------------------------- apply --
cudaError_t apply_term_f64(int64_t n, const int64_t* rowptr, const int32_t* cols, const double* K,
                           const double* eip, unsigned ord, const double* f, double* out, int accumulate,
                           cudaStream_t s);
// (hi, lo) float pair of f[i * stride], i < n
cudaError_t split_f64(const double* f, int64_t n, float2* f2, cudaStream_t s, int64_t stride = 1);
// Dcpse::p2p: out[p][c] = eip_p * sum_q f[q][c] K_pq (reference order)
cudaError_t p2p_f64(int64_t n, const int64_t* rowptr, const int32_t* cols, const double* K, const double* eip,
                    int ncomp, const double* f, double* out, cudaStream_t s);
// Batched FP32 apply with caller-owned arrays: direct (unstaged) kernel,
// lanes per row from nnz / n.
cudaError_t apply_batched_f32(int64_t n, int nout, const int64_t* rowptr, const int32_t* cols, const float* w,
                              int64_t nnz, const float2* f2, double* out, cudaStream_t s);

// Loads the kernels apply_batched_f32 and split_f64 launch onto the current
// device (cudaFuncGetAttributes), so that a later call loads no code.
cudaError_t preload_apply_f32_direct();

// Batched FP32 apply on the sliced ELL layout (SELL-32, rows sorted by length
// within windows of 256): windows [w0, w1) of rows, thread per row.  The
// layout may renumber the rows and columns (perm[position] = list row,
// inv[list row] = position, e.g. a cell order of the particles): its columns
// are then positions, the field pair is read at positions, and outputs go to
// list rows.
struct SellArgs {
    const int32_t* perm;   // position -> list row, or null (identity)
    int64_t n;             // rows
    int64_t nslices;
    const int32_t* srow;   // row of (slice, lane), -1 past the last row
    const int64_t* off;    // [nslices + 1] first entry of each slice
    const int32_t* cols;   // [total] entry-major within a slice
    const float* w;        // [NO][total]
    const __nv_bfloat16* r; // [NO][total] bf16 residuals of the weights, or null
    const float* r32;      // [NO][total] FP32 residuals w64 - w32 (weight pairs), or null
    int64_t total;
    const float2* f2;
    // the field in fixed point (with r32): fx[i] = f_i 2^shift rounded to an
    // integer, shift = fx_meta[1] (kFixedNonFinite: the field holds a NaN or
    // an infinity, and every output is NaN)
    const long long* fx;
    const long long* fx_meta;
    double* out;           // output o of row r at out[o * oos + r * ors]
    int64_t oos, ors;
    int64_t w0, w1;        // windows of 256 rows
    uint32_t comp;
    int no_self;
    // optional: weight-rounding bound of every output of every row,
    // bnd[o * n + r] = sum_q |w_o,pq| |f_q - f_p|, and the call's largest
    // |output| per output as float bits (atomic max; zero it before the call)
    float* bnd;
    unsigned* maxabs;
    int stream;            // evict-first hint on the column, weight and residual streams
    // non-null (device outputs): warps take slices one at a time from this
    // counter (zeroed by apply_sell) and store their rows directly
    unsigned* counter;
};
int64_t sell_slices(int64_t n);
// srow [sell_slices(n) * 32], slen32 [sell_slices(n)], off [sell_slices(n) + 1],
// scan_tmp [scan_tmp_elems(sell_slices(n))]; rows are positions (list row
// perm[position], or the position itself without perm)
cudaError_t sell_order(const int64_t* rowptr, int64_t n, int32_t* srow, int32_t* slen32, int64_t* off,
                       int64_t* scan_tmp, cudaStream_t s, const int32_t* perm = nullptr);
// d_sums[0] = sum over entries |q - p|, d_sums[1] = sum |inv[q] - inv[p]|
cudaError_t sell_locality(const int64_t* rowptr, const int32_t* cols, int64_t n, const int32_t* inv,
                          unsigned long long* d_sums, cudaStream_t s);
cudaError_t invert_perm(const int32_t* perm, int64_t n, int32_t* inv, cudaStream_t s);
// The field in fixed point for the weight pairs' apply: meta[0] = the bits of
// max |f|, meta[1] = shift = 62 - e with max |f| < 2^e (|fx| < 2^62, so that
// differences stay below 2^63), fx[inv[i]] (fx[i] without inv) = f[i] 2^shift
// rounded to the nearest integer; a NaN or an infinity sets shift to
// kFixedNonFinite.
constexpr long long kFixedNonFinite = -(1ll << 40);
cudaError_t fixed_field(const double* f, int64_t n, const int32_t* inv, long long* fx, long long* meta,
                        cudaStream_t s);
// f2[inv[i]] = (hi, lo) of f[i];  g[inv[i]] = f[i]
cudaError_t split_f64_perm(const double* f, int64_t n, const int32_t* inv, float2* f2, cudaStream_t s);
cudaError_t permute_f64(const double* f, int64_t n, const int32_t* inv, double* g, cudaStream_t s);
// Copies into the sliced layout the columns (scols given), the FP32 weights
// (w / sw given) and the bf16 residual streams (r16 / sr16 given); the
// streams asked for must be consecutive in that order.  one_set: the columns
// index the rows' own set.
cudaError_t sell_fill(const int64_t* rowptr, const int32_t* cols, const float* w, const void* r16, int64_t ws,
                      int nout, int64_t n, int one_set, const int32_t* srow, const int64_t* off, int64_t total,
                      int32_t* scols, float* sw, void* sr16, cudaStream_t s, const int32_t* perm = nullptr,
                      const int32_t* inv = nullptr);
cudaError_t apply_sell(const SellArgs& a, int nout, cudaStream_t s);
// FP64 summed weights on the same slices ([nout][total]) and their apply
cudaError_t sell_fill64(const int64_t* rowptr, const double* w, int64_t ws, int nout, int64_t n,
                        const int32_t* srow, const int64_t* off, int64_t total, double* sw, cudaStream_t s,
                        const int32_t* perm = nullptr);
struct Sell64Args {
    const int32_t* perm;    // position -> list row, or null (the field f is then at positions)
    int64_t n, nwin;
    const int32_t* srow;
    const int64_t* off;
    const int32_t* cols;
    const double* w;        // [NO][total]
    int64_t total;
    const double* f;        // field, element i at f[i * fs]
    int64_t fs;
    double* out;            // output o of row r at out[o * oos + r * ors]
    int64_t oos, ors;
    int no_self;
    int stream;             // evict-first hint on the column and weight streams
};
cudaError_t apply_sell64(const Sell64Args& a, int nout, cudaStream_t s);

// FP64 residual correction of a batched FP32 apply where its weight-rounding
// bound exceeds the error budget (see dcpse_budget.cu).
struct BudgetArgs {
    int64_t n;
    const int64_t* rowptr;
    const int32_t* cols;
    const float* r32;          // [nout][ws] FP32 residuals w64 - w32
    const void* r16;           // [nout][ws] bf16 residuals the FP32 apply already added, or null
    int64_t ws;
    const float2* f2;          // the field's float pair (what the FP32 apply read)
    double* out;               // output o of row r at out[o * oos + r * ors]
    int64_t oos, ors;
    const float* bnd;          // [nout][n] bounds of the FP32 apply (unused with flag_all)
    const unsigned* maxabs;    // [nout] largest |output| (float bits)
    double budget;             // relative error budget per output
    double bound_scale;        // error of the FP32 apply <= bound_scale * bnd (2^-24, 2^-32 with r16)
    int flag_all;              // correct every row
    unsigned long long* count; // (row, output) pairs corrected, accumulated, or null
    uint2* list;               // [n] scratch: flagged rows (row, output mask)
    unsigned* list_len;        // its length (zero it before the call)
    const int32_t* inv;        // field pair of list row i at f2[inv[i]], or null (at i)
};
cudaError_t budget_correct(const BudgetArgs& a, int nout, cudaStream_t s);

// Full description of a batched FP32 apply (plan-owned, padded arrays).
struct ApplyF32 {
    int64_t n;
    int nout;
    const int64_t* rowptr;
    const int32_t* cols;   // padded by >= 8 entries past nnz
    const float* w;        // [nout][ws], padded by >= 8 entries past nout*ws
    const void* resid;     // bf16 [nout][ws] residuals (w64 - w32) or null
    int64_t ws;            // stream stride
    int64_t nnz;
    int maxk;              // longest row (sizes the staging buffers)
    const float2* f2;
    double* out;           // [nout][n]
    int* err;              // device error word (bounded waits that ran out)
    int mode;              // 0 automatic (direct), 1 direct, 2 staged, 3 direct x8
    int lanes;             // lanes per row (0 = from the mean row length)
    uint32_t comp;         // outputs taking the compensated FP32 sum (bit per output)
    int no_self;           // interpolation: sum w f_q without the f_p term; f2 on the support set
    int64_t oos, ors;      // output o of row r at out[o * oos + r * ors] (0: n and 1)
    int64_t row0, row1;    // rows [row0, row1) (0, 0: all; a row range needs a direct mode)
};
cudaError_t apply_batched_f32x(const ApplyF32& p, cudaStream_t s);
cudaError_t apply_batched_f64(int64_t n, int nout, const int64_t* rowptr, const int32_t* cols, const double* w,
                              int64_t nnz, const double* f, double* out, cudaStream_t s, int no_self = 0,
                              int64_t oos = 0, int64_t ors = 0, int64_t fs = 0);

// ---------------------------------------------------------- CSR export --
struct MatArgs {
    const int64_t* rowptr;       // neighbour list
    const int32_t* cols;
    const int64_t* rows;         // particles of the exported rows, or null (all)
    int64_t nrows;
    int nterms;                  // terms of the exported output
    const double* K[kMaxTerms];  // their per-term kernels [nnz]
    const double* eip[kMaxTerms];
    double sign[kMaxTerms];      // Dcpse::getSign of each term
    double coeff;
    int64_t nvar, var;           // column index = particle * nvar + var
    const int64_t* out_rowptr;   // [nrows + 1]
    int64_t* out_cols;
    double* out_vals;
};
// entries per exported row (neighbours plus the diagonal unless present)
cudaError_t csr_row_counts(const int64_t* rowptr, const int32_t* cols, const int64_t* rows, int64_t nrows,
                           int32_t* counts, cudaStream_t s);
cudaError_t csr_fill(const MatArgs& a, cudaStream_t s);

// ------------------------------------------------------------- surface --
// support extension along the normals (base particles, then 2 n_count
// virtual particles per base particle) and accumulation of the virtual
// particles' kernels onto their base particles
cudaError_t surface_extend(int dim, const double* base, const double* normals, int64_t nb, int n_count, double spacing,
                           const double* spacings, double* out, cudaStream_t s);
cudaError_t surface_count(const int64_t* rowptr, const int32_t* cols, int64_t n, int64_t nb, int n_count,
                          int32_t* counts, cudaStream_t s);
constexpr int kMaxStreams = kMaxTerms + kMaxOutputs;
struct SurfAcc {
    const int64_t* rowptr;        // list over the extended support
    const int32_t* cols;
    int64_t n, nb;
    int n_count;
    const int64_t* out_rowptr;    // accumulated list over the base particles
    int32_t* out_cols;
    int nst;                      // value streams (per-term kernels, output weights)
    const double* in[kMaxStreams];
    double* out[kMaxStreams];
};
cudaError_t surface_fill(const SurfAcc& a, cudaStream_t s);
// w32 = (float)w64 and the bf16 and FP32 residuals w64 - w32 (r16 and r32
// may be null)
cudaError_t narrow_weights(const double* w64, int64_t m, float* w32, void* r16, cudaStream_t s,
                           float* r32 = nullptr);

// --------------------------------------------------------------- adjoint --
// transposed list: trow[n+1], per entry the source row tsrc and entry index tidx
cudaError_t build_transpose(const int64_t* rowptr, const int32_t* cols, int64_t n, int64_t nnz, int32_t* cnt,
                            int64_t* trow, int64_t* fill, int32_t* tsrc_tmp, int64_t* tidx_tmp, int32_t* tsrc,
                            int64_t* tidx, int64_t* scan_tmp, cudaStream_t s);
cudaError_t row_sums(const int64_t* rowptr, int64_t n, int nout, const double* w64, const float* w32, int64_t ws,
                     double* rs, cudaStream_t s);
cudaError_t vjp_field(const int64_t* trow, const int32_t* tsrc, const int64_t* tidx, int64_t n, int nout,
                      const double* w64, const float* w32, int64_t ws, const double* rs, const double* g, double* out,
                      cudaStream_t s);
// The field VJP on the sliced ELL layout of the transposed list (w: the
// transposed weights of every output on that layout as doubles, FP32 weights
// widened; output o at w + o * total)
struct VjpSellArgs {
    int64_t n, nwin;
    const int32_t* srow;
    const int64_t* off;
    const int32_t* cols;
    const double* w;
    int64_t total;
    const double* rs;   // [nout][n] row sums of the weights
    const double* g;    // [nout][n] cotangents
    double* out;        // [n]
};
cudaError_t vjp_field_sell(const VjpSellArgs& a, int nout, cudaStream_t s);
// wt[o * nnz + t] = w[o * ws + tidx[t]] (w64, else w32 widened)
cudaError_t transpose_outputs(const int64_t* tidx, int64_t nnz, int nout, const double* w64, const float* w32,
                              int64_t ws, double* wt, cudaStream_t s);

struct VjpArgs {
    const AsmTables* tab;
    int64_t n;
    const double* pos;
    const int64_t* rowptr;
    const int32_t* cols;
    Geom geom;
    double h_over_eps;
    const double* eps_fixed;
    const double* f;      // field [n]
    const double* gbar;   // cotangent [noutputs][n]
    double* gentry;       // scratch [nnz][dim]: dPhi_p / dx_pq
};
cudaError_t vjp_positions(const VjpArgs& a, const AsmTables& h, const int64_t* trow, const int64_t* tidx, double* grad,
                          cudaStream_t s);

// ------------------------------------------------- RK4 reaction-diffusion --
template <typename T>
struct RkArgs {
    int64_t n;
    const int64_t* rowptr;
    const int32_t* cols;
    const T* w;                     // Laplacian weights [nnz]
    const T *Yu, *Yv;               // stage input (gathered)
    const T *y0u, *y0v;             // state at the start of the step
    T *accu, *accv;                 // k1 + 2 k2 + 2 k3
    T *outu, *outv;                 // next stage input, or the new state
    double Du, Dv, F, K, dt;
    int stage;                      // 0..3
    void* pack;                     // scratch [n] of (u, v) pairs (float2 / double2) for the gathers
    // the weights on the sliced ELL layout (FP32 state; null: CSR kernel)
    const int32_t* srow;
    const int64_t* soff;
    const int32_t* scols;
    const float* sw;
};
template <typename T>
struct RkAdjArgs {
    int64_t n;
    const int64_t* trow;
    const int32_t* tsrc;
    const T* wT;                    // transposed Laplacian weights
    const T* rs;                    // row sums of the weights
    const T *Yu, *Yv;               // stage state
    const T *kbu, *kbv;             // kbar of this stage
    const T *ybu, *ybv;             // ybar of the step
    T *accu, *accv;                 // ybar_n accumulator (+= Ybar)
    T *next_u, *next_v;             // kbar of the previous stage, or null
    double cy, cY;                  // next kbar = cy ybar + cY Ybar
    double Du, Dv, F, K;
    void* pack;                     // scratch: n (kbar_u, kbar_v) pairs
    // the transposed weights on the sliced ELL layout (FP32; null: CSR kernel)
    const int32_t* srow;
    const int64_t* soff;
    const int32_t* scols;
    const float* sw;
    // fused reverse step: the row's own kbar read from the pairs (kbu, kbv
    // unused), the next kbar written as pairs to pack_out (next_u, next_v
    // unused), and acc_mode 1: acc = ybar + Ybar, 2: ybar = acc + Ybar (in
    // place; acc not written), 0: acc += Ybar
    bool kb_packed;
    void* pack_out;
    int acc_mode;
    T *yb_out_u, *yb_out_v;
};
template <typename T>
cudaError_t rk_stage(const RkArgs<T>& a, int lanes, cudaStream_t s);
template <typename T>
cudaError_t rk_adjoint_stage(const RkAdjArgs<T>& a, int lanes, cudaStream_t s);
// pairs (scale ybar_u, scale ybar_v) into pack: the kbar of a step's last stage
template <typename T>
cudaError_t rk_pack_scaled(const T* ybu, const T* ybv, int64_t n, double scale, void* pack, cudaStream_t s);
template <typename T>
cudaError_t rk_transpose_weights(const int64_t* rowptr, const int64_t* tidx, int64_t n, int64_t nnz, const T* w,
                                 T* wT, T* rs, cudaStream_t s);

int num_sms();

// Rows one full wave of the direct FP32 apply kernel covers (every block
// slot of the GPU busy once), for the given or the automatic lane count.
int64_t f32_rows_per_wave(int64_t n, int64_t nnz, int lanes);

// Records msg as this thread's dcpse_last_error() and returns code.
int set_error(int code, const char* msg);

}  // namespace dcpse
