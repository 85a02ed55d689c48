// dcpse_capi.cu -- the C-ABI of the GB300 DC-PSE path (plan management,
// basis tables, neighbour build, assembly and apply entry points).
//
// Host-side restatement of the reference's basis machinery:
//   MonomialBasis::generateBasis  src/DCPSE/MonomialBasis.hpp:114-157
//   Monomial::getDerivative       src/DCPSE/Monomial.hpp:158-174
//   DcpseRhs::getVector           src/DCPSE/DcpseRhs.hpp:26-60
// The bases are computed once per plan and shipped to the device as tables.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "dcpse_internal.h"

using namespace dcpse;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

#define DCPSE_CK(call)                                                                                  \
    do {                                                                                                \
        cudaError_t e_ = (call);                                                                        \
        if (e_ != cudaSuccess)                                                                          \
            return fail(DCPSE_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));            \
    } while (0)

struct Mono {
    std::array<unsigned, 3> e{0, 0, 0};
    unsigned scalar = 1;
};

// MonomialBasis.hpp:114-157: grid [0, lim)^dim with dimension 0 fastest,
// keep alphaMin <= |m| < lim; lim = |alpha| + r, alphaMin = 1 for even
// |alpha| > 0.
std::vector<Mono> make_basis(int dim, unsigned msum, unsigned r) {
    std::vector<Mono> out;
    unsigned lim = msum + r;
    unsigned amin = (msum % 2 == 0 && msum != 0) ? 1u : 0u;
    long total = 1;
    for (int d = 0; d < dim; ++d) total *= (long)lim;
    for (long lin = 0; lin < total; ++lin) {
        Mono m;
        long t = lin;
        unsigned o = 0;
        for (int d = 0; d < dim; ++d) {
            m.e[d] = (unsigned)(t % lim);
            t /= lim;
            o += m.e[d];
        }
        if (o < lim && o >= amin) out.push_back(m);
    }
    return out;
}

// (D^sig m)(0) * sign, sign = +1 for even |sig| (DcpseRhs.hpp:41-60, with
// Monomial::getDerivative and evaluate at the origin)
double rhs_entry(int dim, const Mono& m, const unsigned* sig) {
    unsigned ord = 0;
    for (int d = 0; d < dim; ++d) ord += sig[d];
    int sign = (ord % 2 == 0) ? 1 : -1;
    unsigned s = m.scalar;
    double val = 1.0;
    for (int d = 0; d < dim; ++d) {
        int target = (int)m.e[d] - (int)sig[d];
        for (int k = (int)m.e[d]; k > target && k >= 0; --k) s *= (unsigned)k;
        unsigned ne = (unsigned)std::max(target, 0);
        val = val * (ne == 0 ? 1.0 : 0.0);
    }
    return sign * ((double)s * val);
}

__global__ void status_summary_kernel(const int32_t* st, int64_t n, unsigned long long* out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if (st[i] != 0) {
            atomicAdd(&out[0], 1ull);
            atomicMin(&out[1], (unsigned long long)i);
        }
    }
}

// Checks a caller-supplied CSR list: rowptr[0] = 0, rowptr[n] = nnz, rows
// non-decreasing, every column in [0, n).  bad[0] counts violations.
__global__ void csr_check_kernel(const int64_t* rowptr, const int32_t* cols, int64_t n, int64_t nnz, int64_t ncols,
                                 unsigned long long* bad) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t t0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    for (int64_t i = t0; i < n; i += stride)
        if (rowptr[i + 1] < rowptr[i]) atomicAdd(bad, 1ull);
    for (int64_t j = t0; j < nnz; j += stride)
        if (cols[j] < 0 || (int64_t)cols[j] >= ncols) atomicAdd(bad, 1ull);
    if (t0 == 0 && (rowptr[0] != 0 || rowptr[n] != nnz)) atomicAdd(bad, 1ull);
}

__global__ void index_check_kernel(const int64_t* idx, int64_t m, int64_t n, unsigned long long* bad) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
        if (idx[i] < 0 || idx[i] >= n) atomicAdd(bad, 1ull);
}

// Host-buffer applies move the field up and the outputs back in row chunks
// overlapped with the apply of other chunks.  Chunk boundaries fall on whole
// waves of the apply kernel's grid (a chunk of 1.7 waves would run its second
// wave two thirds full), with sizes tapering at both ends, 1 1 2 4 4 4 4 4 4
// 2 1 1 32nds of the waves: small first chunks start the apply after a short
// upload, small last chunks leave a short copy after the last apply.
constexpr int kHostChunks = 12;
constexpr int64_t kHostChunkMinRows = 65536;
struct ChunkBounds {
    int nch;
    int64_t b[kHostChunks + 1];  // chunk c = rows [b[c], b[c + 1])
};

ChunkBounds make_chunk_bounds(int64_t n, int64_t rows_per_wave) {
    static const int cum[kHostChunks + 1] = {0, 1, 2, 4, 8, 12, 16, 20, 24, 28, 30, 31, 32};
    ChunkBounds c{};
    const int64_t waves = (n + rows_per_wave - 1) / rows_per_wave;
    if (waves <= kHostChunks) {
        c.nch = (int)std::max<int64_t>(waves, 1);
        for (int i = 0; i <= c.nch; ++i) c.b[i] = std::min(n, (int64_t)i * rows_per_wave);
        c.b[c.nch] = n;
        return c;
    }
    c.nch = kHostChunks;
    // bounds on whole windows of 256 rows (the sliced ELL kernel's unit)
    for (int i = 0; i <= kHostChunks; ++i) c.b[i] = std::min(n, (n * cum[i] / 32) & ~int64_t(255));
    c.b[kHostChunks] = n;
    return c;
}

// largest field index each row chunk reads (its neighbours and itself)
__global__ void chunk_reach_kernel(const int64_t* rowptr, const int32_t* cols, int64_t n, ChunkBounds cb,
                                   unsigned long long* reach) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        int c = 0;
        while (c + 1 < cb.nch && cb.b[c + 1] <= r) ++c;
        int64_t m = r;
        for (int64_t j = rowptr[r]; j < rowptr[r + 1]; ++j) m = max(m, (int64_t)cols[j]);
        atomicMax(&reach[c], (unsigned long long)m);
    }
}

__global__ void row_max_kernel(const int64_t* rowptr, int64_t n, int* maxk) {
    int m = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        m = max(m, (int)(rowptr[i + 1] - rowptr[i]));
    atomicMax(maxk, m);
}

// Entries of padding after the column and FP32 weight arrays: the staged
// apply copies 16-byte aligned windows that may end up to 7 entries past the
// last used one.
constexpr int64_t kPad = 8;

// Largest scratch of one assembly batch; larger clouds are assembled in
// batches of particles (the result does not depend on the batch size).
constexpr int64_t kAsmScratchBytes = int64_t(512) << 20;

template <typename T>
cudaError_t dalloc(T** p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    return cudaMalloc((void**)p, count * sizeof(T));
}

template <typename T>
void dfree(T*& p) {
    if (p) cudaFree((void*)p);
    p = nullptr;
}

}  // namespace

int dcpse::set_error(int code, const char* msg) { return fail(code, msg); }

struct KernelTimer {
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev;
    size_t used = 0;
};

struct dcpse_plan_s {
    // optional event timing per kernel id
    bool timing = false;
    KernelTimer timers[DCPSE_K_COUNT];
    void tstart(int k, cudaStream_t on = nullptr) {
        if (!timing) return;
        KernelTimer& T = timers[k];
        if (T.used == T.ev.size()) {
            cudaEvent_t a, b;
            cudaEventCreate(&a);
            cudaEventCreate(&b);
            T.ev.emplace_back(a, b);
        }
        cudaEventRecord(T.ev[T.used].first, on ? on : stream);
    }
    void tstop(int k, cudaStream_t on = nullptr) {
        if (!timing) return;
        KernelTimer& T = timers[k];
        cudaEventRecord(T.ev[T.used].second, on ? on : stream);
        T.used++;
    }
    void free_timers() {
        for (auto& T : timers) {
            for (auto& p : T.ev) {
                cudaEventDestroy(p.first);
                cudaEventDestroy(p.second);
            }
            T.ev.clear();
            T.used = 0;
        }
    }
    int dim = 0;
    unsigned order = 2;
    double hoe = 0.9;
    int nout = 0, nterms = 0;
    std::vector<int> term_output;
    std::vector<std::array<unsigned, 3>> sigs;
    std::vector<int> term_group;
    std::vector<std::vector<Mono>> gbasis;
    AsmTables* htab = nullptr;  // host copy
    AsmTables* dtab = nullptr;  // device copy
    cudaStream_t stream = nullptr;
    bool has_box = false;
    double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    int per[3] = {0, 0, 0};
    // support set of the columns (PPInterpolation, two-set Dcpse); null: the
    // domain set itself, with or without the particle itself in its list
    const double* sup_pos = nullptr;
    int64_t n_sup = 0;
    int self_skip = 1;
    bool two_set() const { return sup_pos != nullptr; }
    // surface DC-PSE: normals (and optional per-particle spacings) of the base
    // support particles; the extended support is plan-owned
    const double* surf_normals = nullptr;
    const double* surf_spacings = nullptr;
    double surf_spacing = 0.0;
    int surf_count = 0;
    double* surf_ext = nullptr;
    int64_t surf_nb = 0;          // base particles of the extended support
    bool surf_pending = false;    // the list refers to the extended support
    bool surface() const { return surf_normals != nullptr; }
    // neighbour list
    int64_t n = -1, nnz = 0;
    int maxk = 0;
    int64_t* rowptr = nullptr;
    int32_t* cols = nullptr;
    // assembly results
    bool assembled = false;
    int flags = 0;
    double* eps = nullptr;
    int32_t* status = nullptr;
    double* eip_group = nullptr;
    double* k_term = nullptr;
    double* w64 = nullptr;
    float* w32 = nullptr;
    void* r16 = nullptr;  // bf16 residuals of w32
    float* r32 = nullptr;  // FP32 residuals w64 - w32 (budget-driven correction)
    // budget-driven FP32 apply: relative error budget per output, the FP32
    // kernel's bounds [nout][n], the call's largest |output| per output and
    // the (row, output) pairs corrected since the last reset
    double budget = 1e-6;
    int budget_pass = DCPSE_F32;  // first pass: DCPSE_F32 or DCPSE_F32_RESID (adds the bf16 streams)
    float* bnd = nullptr;
    uint2* blist = nullptr;  // rows to correct (scratch)
    int64_t bnd_len = 0;
    unsigned* maxabs = nullptr;  // [kMaxOutputs] largest |output|, then the list length
    unsigned long long* budget_count = nullptr;
    unsigned* slice_counter = nullptr;  // the warp-scheduled sliced kernels' slice counter
    double sell_idle = 0.0;  // share of warp time the window barrier would idle on the sliced layout
    unsigned long long* summary = nullptr;  // [count, first]
    int* d_err = nullptr;                   // set by kernels whose bounded wait ran out
    int apply_lanes = 0, apply_mode = 0;
    bool asm_tc = false;  // the last assembly's Gram products ran on the tensor cores
    int asm_bin_width = 0, asm_warps = 4, asm_qr_lanes = 0;
    double* asm_scratch = nullptr;  // assembly batch scratch
    int64_t asm_scratch_bytes = 0;
    double* qr_ws = nullptr;        // global QR work space of bases too large for shared memory
    int64_t qr_ws_bytes = 0;
    int32_t* korder = nullptr;  // k-binned particle order of the current list
    int korder_width = 0;
    // transposed list and weight row sums (adjoint), built on demand
    int64_t* t_row = nullptr;
    int32_t* t_src = nullptr;
    int64_t* t_idx = nullptr;
    double* rowsum = nullptr;
    int rowsum_prec = -1;
    double* gentry = nullptr;
    // transposed Laplacian weights of output 0 for the RK4 adjoint, and the
    // FP32 ones on a sliced ELL layout of the transposed list
    float *wT32 = nullptr, *rs32 = nullptr;
    double *wT64 = nullptr, *rs64 = nullptr;
    int32_t *tsell_row = nullptr, *tsell_cols = nullptr;
    int64_t* tsell_off = nullptr;
    float* tsell_w = nullptr;
    void free_tsell() {
        dfree(tsell_row);
        dfree(tsell_cols);
        dfree(tsell_off);
        dfree(tsell_w);
    }
    // the transposed list on a sliced ELL layout with the weights of every
    // output gathered into it (the field VJP), per precision
    int32_t *vsell_row = nullptr, *vsell_cols = nullptr;
    int64_t* vsell_off = nullptr;
    int64_t vsell_total = 0;
    bool vsell_no_room = false;
    double* vsell_w64 = nullptr;
    double* vsell_w32 = nullptr;  // the FP32 weights, widened
    void free_vsell_weights() {
        dfree(vsell_w64);
        dfree(vsell_w32);
    }
    void free_vsell() {
        dfree(vsell_row);
        dfree(vsell_cols);
        dfree(vsell_off);
        vsell_total = 0;
        vsell_no_room = false;
        free_vsell_weights();
    }
    void free_transpose() {
        free_vsell();
        dfree(korder);
        korder_width = 0;
        dfree(t_row);
        dfree(t_src);
        dfree(t_idx);
        dfree(rowsum);
        dfree(gentry);
        dfree(wT32);
        dfree(rs32);
        dfree(wT64);
        dfree(rs64);
        free_tsell();
        rowsum_prec = -1;
    }
    // RK4 stage scratch: (u, v) pairs, as doubles
    double* rk_pack = nullptr;
    int64_t rk_pack_n = 0;
    // apply scratch
    float2* f2 = nullptr;
    int64_t f2_len = 0;
    long long* fx_meta = nullptr;  // [2] of the fixed-point field (the weight pairs' apply)
    // host-buffer applies: the field arrives in pieces on h2d_stream, row
    // chunks start once the pieces they read have arrived, and their outputs
    // go back on copy_stream while later chunks run
    cudaStream_t copy_stream = nullptr, h2d_stream = nullptr, apply2_stream = nullptr;
    cudaEvent_t chunk_ev[kHostChunks] = {};
    cudaEvent_t piece_ev[kHostChunks] = {};
    int64_t chunk_reach[kHostChunks] = {};
    ChunkBounds chunks{};                // row chunks the reaches are for
    int64_t list_version = 0;            // bumped whenever the neighbour list changes
    int64_t reach_version = -1;          // list version the reaches were computed for
    double* hf = nullptr;    // device copy of a host field (host apply), hf_len values
    double* hout = nullptr;  // device outputs for host apply, nout * hf_len values
    int64_t hf_len = 0;      // particles hf and hout were sized for (the list may change n)

    // Z-order of the particles' cells from the neighbour build (one set
    // only): cell_order[k] = the particle in position k
    int32_t* cell_order = nullptr;
    int reorder = 0;  // -1: keep the list's numbering, 0: automatic, 1: cell order
    int reorder_order = 0;  // the renumbering order built with the list (0 Z-order of cells, 1 row-major)
    // the FP32 output weights on the sliced ELL layout (built on first use);
    // with sell_perm the layout is in cell order (sell_perm = cell_order,
    // sell_inv its inverse)
    const int32_t* sell_perm = nullptr;
    int32_t* sell_inv = nullptr;
    double* fperm = nullptr;  // the FP64 field at positions (FP64 applies on a renumbered layout)
    int64_t fperm_len = 0;
    unsigned long long loc_sum[2] = {0, 0};  // locality of the list / cell numbering (sum |q - p|)
    int32_t* sell_row = nullptr;
    int64_t* sell_off = nullptr;
    int32_t* sell_cols = nullptr;
    float* sell_w = nullptr;
    void* sell_r = nullptr;  // bf16 residuals on the same layout (with r16)
    float* sell_r32 = nullptr;  // FP32 residuals on the same layout (with r32: the weight pairs)
    double* sell_w64 = nullptr;  // FP64 summed weights on the same layout (with w64)
    int64_t sell_total = 0;
    bool sell_no_room = false;  // the copy did not fit in device memory: CSR kernels only
    void free_sell() {
        sell_perm = nullptr;
        dfree(sell_inv);
        dfree(fperm);
        fperm_len = 0;
        dfree(sell_row);
        dfree(sell_off);
        dfree(sell_cols);
        dfree(sell_w);
        dfree(sell_w64);
        if (sell_r) cudaFree(sell_r);
        sell_r = nullptr;
        dfree(sell_r32);
        sell_total = 0;
        sell_no_room = false;
    }
    void free_assembly() {
        free_sell();
        dfree(eps);
        dfree(status);
        dfree(eip_group);
        dfree(k_term);
        dfree(w64);
        dfree(w32);
        if (r16) cudaFree(r16);
        r16 = nullptr;
        dfree(r32);
        dfree(bnd);
        dfree(blist);
        bnd_len = 0;
        dfree(rowsum);
        rowsum_prec = -1;
        free_vsell_weights();
        dfree(wT32);
        dfree(rs32);
        dfree(wT64);
        dfree(rs64);
        free_tsell();
        assembled = false;
    }
    void free_all() {
        free_assembly();
        free_transpose();
        dfree(rowptr);
        dfree(cols);
        dfree(cell_order);
        dfree(f2);
        dfree(fx_meta);
        dfree(hf);
        dfree(hout);
        hf_len = 0;
        dfree(summary);
        dfree(d_err);
        dfree(maxabs);
        dfree(budget_count);
        dfree(slice_counter);
        dfree(asm_scratch);
        asm_scratch_bytes = 0;
        dfree(qr_ws);
        qr_ws_bytes = 0;
        dfree(rk_pack);
        rk_pack_n = 0;
        if (copy_stream) {
            cudaStreamSynchronize(copy_stream);
            cudaStreamSynchronize(h2d_stream);
            for (auto* evs : {chunk_ev, piece_ev})
                for (int i = 0; i < kHostChunks; ++i) {
                    if (evs[i]) cudaEventDestroy(evs[i]);
                    evs[i] = nullptr;
                }
            cudaStreamSynchronize(apply2_stream);
            cudaStreamDestroy(copy_stream);
            cudaStreamDestroy(h2d_stream);
            cudaStreamDestroy(apply2_stream);
            copy_stream = nullptr;
            h2d_stream = nullptr;
            apply2_stream = nullptr;
        }
        reach_version = -1;
        dfree(surf_ext);
        dfree(dtab);
        delete htab;
        htab = nullptr;
        free_timers();
    }
};

namespace {

// Monomial program of the union basis (see AsmTables::prog).  Powers follow
// ipow's square-and-multiply steps, keyed by the exponent reached, so every
// intermediate power is computed once; monomials multiply their non-unit
// factors left to right in dimension order, sharing common prefixes.
int build_program(AsmTables* T) {
    const int dim = T->dim;
    T->nprog = 0;
    auto op = [&](int x, int y) -> int {
        if (dim + 1 + T->nprog >= kMaxSlots) return -1;
        T->prog[T->nprog][0] = (unsigned char)x;
        T->prog[T->nprog][1] = (unsigned char)y;
        return dim + 1 + T->nprog++;
    };
    std::map<std::pair<int, int>, int> pw;  // (d, exponent) -> slot
    auto power = [&](int d, int e) -> int {
        int top = 0;
        while ((e >> (top + 1)) != 0) ++top;
        int cur = d, p = 1;
        for (int b = top - 1; b >= 0 && cur >= 0; --b) {
            p = 2 * p;
            auto it = pw.find({d, p});
            cur = (it != pw.end()) ? it->second : (pw[{d, p}] = op(cur, cur));
            if (cur >= 0 && ((e >> b) & 1)) {
                p = p + 1;
                auto jt = pw.find({d, p});
                cur = (jt != pw.end()) ? jt->second : (pw[{d, p}] = op(cur, d));
            }
        }
        return cur;
    };
    std::map<std::vector<int>, int> prod;  // factor slots -> slot of their product
    for (int j = 0; j < T->nu; ++j) {
        std::vector<int> f;
        for (int d = 0; d < dim; ++d)
            if (T->uexp[j][d] > 0) f.push_back(power(d, T->uexp[j][d]));
        for (int x : f)
            if (x < 0) return -1;
        int cur = dim;  // the constant 1.0
        if (!f.empty()) {
            cur = f[0];
            std::vector<int> key{f[0]};
            for (size_t m = 1; m < f.size() && cur >= 0; ++m) {
                key.push_back(f[m]);
                auto it = prod.find(key);
                cur = (it != prod.end()) ? it->second : (prod[key] = op(cur, f[m]));
            }
        }
        if (cur < 0) return -1;
        T->uslot[j] = (unsigned char)cur;
    }
    T->nslots = dim + 1 + T->nprog;
    return 0;
}

int build_tables(dcpse_plan_s* P) {
    AsmTables* T = P->htab;
    std::memset(T, 0, sizeof(AsmTables));
    T->dim = P->dim;
    // groups by |alpha| (the basis depends on |alpha| and the order only)
    std::vector<unsigned> gkey;
    P->term_group.assign(P->nterms, 0);
    for (int t = 0; t < P->nterms; ++t) {
        unsigned ms = 0;
        for (int d = 0; d < P->dim; ++d) ms += P->sigs[t][d];
        auto it = std::find(gkey.begin(), gkey.end(), ms);
        if (it == gkey.end()) {
            gkey.push_back(ms);
            P->term_group[t] = (int)gkey.size() - 1;
        } else {
            P->term_group[t] = (int)(it - gkey.begin());
        }
    }
    if ((int)gkey.size() > kMaxGroups) return fail(DCPSE_ERR_CAPACITY, "too many distinct operator orders in one plan");
    T->ngroups = (int)gkey.size();
    P->gbasis.clear();
    std::vector<std::array<unsigned, 3>> uni;
    for (int g = 0; g < T->ngroups; ++g) {
        auto B = make_basis(P->dim, gkey[g], P->order);
        if ((int)B.size() > kMaxBasis) return fail(DCPSE_ERR_CAPACITY, "basis larger than supported");
        T->gn[g] = (int)B.size();
        T->gord[g] = (int)gkey[g];
        for (size_t i = 0; i < B.size(); ++i) {
            auto it = std::find(uni.begin(), uni.end(), B[i].e);
            int ui;
            if (it == uni.end()) {
                uni.push_back(B[i].e);
                ui = (int)uni.size() - 1;
            } else {
                ui = (int)(it - uni.begin());
            }
            if (ui >= kMaxUnion) return fail(DCPSE_ERR_CAPACITY, "union basis larger than supported");
            T->gidx[g][i] = (unsigned char)ui;
        }
        P->gbasis.push_back(B);
    }
    T->nu = (int)uni.size();
    int maxe = 0;
    for (int j = 0; j < T->nu; ++j)
        for (int d = 0; d < P->dim; ++d) {
            T->uexp[j][d] = (unsigned char)uni[j][d];
            maxe = std::max(maxe, (int)uni[j][d]);
        }
    T->maxexp = maxe + 1;
    if (T->maxexp > kMaxExp) return fail(DCPSE_ERR_CAPACITY, "monomial degree larger than supported");
    if (build_program(T) != 0) return fail(DCPSE_ERR_CAPACITY, "monomial program larger than supported");
    // Gram entries needed by some group
    std::vector<std::pair<int, int>> pairs;
    for (int g = 0; g < T->ngroups; ++g)
        for (int i = 0; i < T->gn[g]; ++i)
            for (int j = 0; j < T->gn[g]; ++j) {
                int a = T->gidx[g][i], b = T->gidx[g][j];
                if (a <= b) pairs.emplace_back(a, b);
            }
    std::sort(pairs.begin(), pairs.end());
    pairs.erase(std::unique(pairs.begin(), pairs.end()), pairs.end());
    if ((int)pairs.size() > kMaxPairs) return fail(DCPSE_ERR_CAPACITY, "too many Gram entries");
    T->npairs = (int)pairs.size();
    for (int a = 0; a < kMaxUnion; ++a)
        for (int b = 0; b < kMaxUnion; ++b) T->upair[a][b] = -1;
    for (int e = 0; e < T->npairs; ++e) {
        T->pi[e] = (unsigned char)pairs[e].first;
        T->pj[e] = (unsigned char)pairs[e].second;
        T->upair[pairs[e].first][pairs[e].second] = (short)e;
    }
    // right-hand sides
    T->nterms = P->nterms;
    T->noutputs = P->nout;
    for (int t = 0; t < P->nterms; ++t) {
        T->term_group[t] = P->term_group[t];
        T->term_output[t] = P->term_output[t];
    }
    for (int g = 0; g < T->ngroups; ++g) {
        const auto& B = P->gbasis[g];
        for (int t = 0; t < P->nterms; ++t) {
            if (P->term_group[t] != g) continue;
            int r = T->nterm_rhs[g]++;
            if (r >= kMaxRhs) return fail(DCPSE_ERR_CAPACITY, "too many terms of one order");
            T->term_of_rhs[g][r] = t;
            for (size_t i = 0; i < B.size(); ++i) T->b_term[g][r][i] = rhs_entry(P->dim, B[i], P->sigs[t].data());
        }
        for (int o = 0; o < P->nout; ++o) {
            bool touches = false;
            for (int t = 0; t < P->nterms; ++t) touches |= (P->term_output[t] == o && P->term_group[t] == g);
            if (!touches) continue;
            int r = T->nout_rhs[g]++;
            if (r >= kMaxRhs) return fail(DCPSE_ERR_CAPACITY, "too many outputs of one order");
            T->out_of_rhs[g][r] = o;
            for (size_t i = 0; i < B.size(); ++i) {
                double v = 0.0;
                for (int t = 0; t < P->nterms; ++t)
                    if (P->term_output[t] == o && P->term_group[t] == g)
                        v = v + rhs_entry(P->dim, B[i], P->sigs[t].data());
                T->b_out[g][r][i] = v;
            }
        }
    }
    return DCPSE_OK;
}

Geom plan_geom(const dcpse_plan_s* P) {
    Geom g{};
    for (int d = 0; d < kMaxDim; ++d) {
        g.per[d] = (P->has_box && d < P->dim) ? P->per[d] : 0;
        g.L[d] = P->hi[d] - P->lo[d];
        g.half[d] = 0.5 * g.L[d];
    }
    return g;
}

int check_plan(dcpse_plan_t* P) {
    if (!P) return fail(DCPSE_ERR_ARG, "null plan");
    return DCPSE_OK;
}

// Derivative applies, adjoints and the RK4 stages read f on the rows and on
// the columns: they need the domain set to be its own support.
int check_single_set(dcpse_plan_t* P) {
    if (P->two_set())
        return fail(DCPSE_ERR_STATE, "this operation needs a single particle set (use dcpse_p2p on two sets)");
    return DCPSE_OK;
}

// FP32 split of n field values (stride apart) into the plan's scratch; with
// inv (stride 1) value i goes to position inv[i] (a renumbered layout)
int split_into_plan(dcpse_plan_t* P, const double* d_f, int64_t n, int64_t stride, const int32_t* inv = nullptr) {
    if (P->f2_len < n) {
        dfree(P->f2);
        P->f2_len = 0;
        DCPSE_CK(dalloc(&P->f2, (size_t)n));
        P->f2_len = n;
    }
    P->tstart(DCPSE_K_SPLIT);
    cudaError_t e = inv ? split_f64_perm(d_f, n, inv, P->f2, P->stream) : split_f64(d_f, n, P->f2, P->stream, stride);
    P->tstop(DCPSE_K_SPLIT);
    DCPSE_CK(e);
    return DCPSE_OK;
}

// The field in fixed point into the plan's scratch (the float-pair buffer,
// 8 bytes per value either way), at positions when inv is given.
int fixed_into_plan(dcpse_plan_t* P, const double* d_f, const int32_t* inv) {
    static_assert(sizeof(float2) == sizeof(long long), "the fixed-point field shares the pair buffer");
    if (P->f2_len < P->n) {
        dfree(P->f2);
        P->f2_len = 0;
        DCPSE_CK(dalloc(&P->f2, (size_t)P->n));
        P->f2_len = P->n;
    }
    if (!P->fx_meta) DCPSE_CK(dalloc(&P->fx_meta, 2));
    P->tstart(DCPSE_K_SPLIT);
    cudaError_t e = fixed_field(d_f, P->n, inv, reinterpret_cast<long long*>(P->f2), P->fx_meta, P->stream);
    P->tstop(DCPSE_K_SPLIT);
    DCPSE_CK(e);
    return DCPSE_OK;
}

// SurfaceDcpse::accumulateAndDeleteNormalParticles on the plan's arrays: the
// list over the extended support becomes a list over the base particles,
// the per-term kernels and FP64 output weights are accumulated, FP32 weights
// (and residuals) are derived from the accumulated FP64 weights.
int surface_finish(dcpse_plan_s* P, int flags) {
    cudaStream_t s = P->stream;
    const int64_t n = P->n, nnz = P->nnz;
    int32_t* counts = nullptr;
    int64_t *rp2 = nullptr, *tmp = nullptr;
    int32_t* cols2 = nullptr;
    double *k2 = nullptr, *w2 = nullptr;
    auto cleanup = [&]() {
        dfree(counts);
        dfree(tmp);
        dfree(rp2);
        dfree(cols2);
        dfree(k2);
        dfree(w2);
    };
    cudaError_t e = dalloc(&counts, (size_t)std::max<int64_t>(n, 1));
    if (e == cudaSuccess) e = dalloc(&tmp, (size_t)scan_tmp_elems(std::max<int64_t>(n, 1)));
    if (e == cudaSuccess) e = dalloc(&rp2, (size_t)n + 1);
    if (e == cudaSuccess) e = surface_count(P->rowptr, P->cols, n, P->surf_nb, P->surf_count, counts, s);
    if (e == cudaSuccess) e = exclusive_scan_i32(counts, n, rp2, tmp, s);
    int64_t nnz2 = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&nnz2, rp2 + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = dalloc(&cols2, (size_t)nnz2 + kPad);
    if (e == cudaSuccess && nnz2 + kPad > 0) e = cudaMemsetAsync(cols2, 0, sizeof(int32_t) * (nnz2 + kPad), s);
    if (e == cudaSuccess && P->k_term) e = dalloc(&k2, (size_t)P->nterms * std::max<int64_t>(nnz2, 1));
    if (e == cudaSuccess && P->w64) e = dalloc(&w2, (size_t)P->nout * std::max<int64_t>(nnz2, 1));
    if (e != cudaSuccess) {
        cleanup();
        return fail(DCPSE_ERR_CUDA, std::string("surface accumulation: ") + cudaGetErrorString(e));
    }
    SurfAcc a{};
    a.rowptr = P->rowptr;
    a.cols = P->cols;
    a.n = n;
    a.nb = P->surf_nb;
    a.n_count = P->surf_count;
    a.out_rowptr = rp2;
    a.out_cols = cols2;
    if (k2)
        for (int t = 0; t < P->nterms; ++t) {
            a.in[a.nst] = P->k_term + (size_t)t * nnz;
            a.out[a.nst++] = k2 + (size_t)t * nnz2;
        }
    if (w2)
        for (int o = 0; o < P->nout; ++o) {
            a.in[a.nst] = P->w64 + (size_t)o * nnz;
            a.out[a.nst++] = w2 + (size_t)o * nnz2;
        }
    e = surface_fill(a, s);
    if (e != cudaSuccess) {
        cleanup();
        return fail(DCPSE_ERR_CUDA, std::string("surface accumulation: ") + cudaGetErrorString(e));
    }
    // the plan now holds the accumulated operator over the base particles
    P->free_transpose();
    P->free_sell();
    dfree(P->cell_order);
    dfree(P->rowptr);
    P->list_version++;
    dfree(P->cols);
    dfree(P->k_term);
    dfree(P->w64);
    dfree(P->w32);
    if (P->r16) cudaFree(P->r16);
    P->r16 = nullptr;
    dfree(P->r32);
    P->rowptr = rp2;
    P->cols = cols2;
    P->k_term = k2;
    P->w64 = w2;
    rp2 = nullptr;
    cols2 = nullptr;
    k2 = nullptr;
    w2 = nullptr;
    cleanup();
    P->nnz = nnz2;
    P->surf_pending = false;
    int* mk = nullptr;
    DCPSE_CK(dalloc(&mk, 1));
    DCPSE_CK(cudaMemsetAsync(mk, 0, sizeof(int), s));
    if (n > 0) row_max_kernel<<<std::max(1, std::min(num_sms() * 4, (int)((n + 255) / 256))), 256, 0, s>>>(P->rowptr, n, mk);
    int hk = 0;
    DCPSE_CK(cudaMemcpyAsync(&hk, mk, sizeof(int), cudaMemcpyDeviceToHost, s));
    DCPSE_CK(cudaStreamSynchronize(s));
    dfree(mk);
    P->maxk = hk;
    if (flags & DCPSE_STORE_OUT_F32) {
        DCPSE_CK(dalloc(&P->w32, (size_t)P->nout * nnz2 + kPad));
        DCPSE_CK(cudaMemsetAsync(P->w32, 0, sizeof(float) * ((size_t)P->nout * nnz2 + kPad), s));
        if (flags & DCPSE_STORE_OUT_F32_RESID) {
            DCPSE_CK(cudaMalloc(&P->r16, ((size_t)P->nout * nnz2 + kPad) * 2));
            DCPSE_CK(cudaMemsetAsync(P->r16, 0, ((size_t)P->nout * nnz2 + kPad) * 2, s));
        }
        if (flags & DCPSE_STORE_OUT_F32_CORR) DCPSE_CK(dalloc(&P->r32, (size_t)P->nout * nnz2 + kPad));
        DCPSE_CK(narrow_weights(P->w64, (int64_t)P->nout * nnz2, P->w32, P->r16, s, P->r32));
        if (!(flags & DCPSE_STORE_OUT_F64)) dfree(P->w64);
    }
    return DCPSE_OK;
}

}  // namespace

extern "C" {

const char* dcpse_last_error(void) { return g_err.c_str(); }

int dcpse_version(void) { return 1; }

int dcpse_plan_create(dcpse_plan_t** plan, int dim, int n_outputs, const int* terms_per_output,
                      const unsigned* signatures, unsigned order, double h_over_eps) {
    if (!plan) return fail(DCPSE_ERR_ARG, "plan is NULL");
    *plan = nullptr;
    if (dim < 1 || dim > 3) return fail(DCPSE_ERR_ARG, "dim must be 1, 2 or 3");
    if (n_outputs < 1 || n_outputs > kMaxOutputs) return fail(DCPSE_ERR_CAPACITY, "1..8 outputs per plan");
    if (!terms_per_output || !signatures) return fail(DCPSE_ERR_ARG, "NULL terms/signatures");
    if (!(h_over_eps > 0.0)) return fail(DCPSE_ERR_ARG, "h_over_eps must be > 0");
    if (order < 1) return fail(DCPSE_ERR_ARG, "convergence order must be >= 1");
    auto* P = new dcpse_plan_s();
    P->dim = dim;
    P->order = order;
    P->hoe = h_over_eps;
    P->nout = n_outputs;
    int t = 0;
    for (int o = 0; o < n_outputs; ++o) {
        if (terms_per_output[o] < 1) {
            delete P;
            return fail(DCPSE_ERR_ARG, "each output needs at least one term");
        }
        for (int i = 0; i < terms_per_output[o]; ++i, ++t) {
            std::array<unsigned, 3> s{0, 0, 0};
            for (int d = 0; d < dim; ++d) s[d] = signatures[(size_t)t * dim + d];
            P->sigs.push_back(s);
            P->term_output.push_back(o);
        }
    }
    P->nterms = t;
    if (t > kMaxTerms) {
        delete P;
        return fail(DCPSE_ERR_CAPACITY, "too many terms in one plan");
    }
    P->htab = new AsmTables();
    int rc = build_tables(P);
    if (rc != DCPSE_OK) {
        P->free_all();
        delete P;
        return rc;
    }
    cudaError_t e = dalloc(&P->dtab, 1);
    if (e == cudaSuccess) e = cudaMemcpy(P->dtab, P->htab, sizeof(AsmTables), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = dalloc(&P->summary, 2);
    if (e == cudaSuccess) e = dalloc(&P->d_err, 1);
    if (e == cudaSuccess) e = cudaMemset(P->d_err, 0, sizeof(int));
    if (e != cudaSuccess) {
        P->free_all();
        delete P;
        return fail(DCPSE_ERR_CUDA, std::string("plan allocation: ") + cudaGetErrorString(e));
    }
    *plan = P;
    return DCPSE_OK;
}

int dcpse_plan_destroy(dcpse_plan_t* P) {
    if (!P) return DCPSE_OK;
    if (P->stream) cudaStreamSynchronize(P->stream);
    P->free_all();
    delete P;
    return DCPSE_OK;
}

int dcpse_plan_set_stream(dcpse_plan_t* P, void* stream) {
    if (int rc = check_plan(P)) return rc;
    P->stream = (cudaStream_t)stream;
    return DCPSE_OK;
}

int dcpse_plan_set_box(dcpse_plan_t* P, const double* lo, const double* hi, const int* periodic) {
    if (int rc = check_plan(P)) return rc;
    if (!lo || !hi) {
        P->has_box = false;
        return DCPSE_OK;
    }
    for (int d = 0; d < P->dim; ++d) {
        if (!(hi[d] > lo[d])) return fail(DCPSE_ERR_ARG, "box hi must exceed lo");
        P->lo[d] = lo[d];
        P->hi[d] = hi[d];
        P->per[d] = periodic ? (periodic[d] != 0) : 0;
    }
    P->has_box = true;
    return DCPSE_OK;
}

int dcpse_plan_set_support(dcpse_plan_t* P, const double* d_pos_support, int64_t n_support, int self_skip) {
    if (int rc = check_plan(P)) return rc;
    if (d_pos_support && n_support < 0) return fail(DCPSE_ERR_ARG, "bad support set size");
    if (d_pos_support && n_support >= (int64_t)INT32_MAX) return fail(DCPSE_ERR_CAPACITY, "at most 2^31-1 particles");
    // the neighbour list and everything assembled on it refer to the old sets
    P->free_assembly();
    P->free_transpose();
    dfree(P->rowptr);
    P->list_version++;
    dfree(P->cols);
    P->n = -1;
    P->nnz = 0;
    P->maxk = 0;
    P->sup_pos = d_pos_support;
    P->n_sup = d_pos_support ? n_support : 0;
    P->self_skip = self_skip ? 1 : 0;
    return DCPSE_OK;
}

int dcpse_plan_set_surface(dcpse_plan_t* P, const double* d_normals, int n_count, double n_spacing,
                           const double* d_n_spacings) {
    if (int rc = check_plan(P)) return rc;
    if (d_normals && n_count < 1) return fail(DCPSE_ERR_ARG, "n_count must be >= 1");
    if (d_normals && !d_n_spacings && !(n_spacing > 0.0)) return fail(DCPSE_ERR_ARG, "n_spacing must be > 0");
    P->free_assembly();
    P->free_transpose();
    dfree(P->rowptr);
    P->list_version++;
    dfree(P->cols);
    dfree(P->surf_ext);
    P->n = -1;
    P->nnz = 0;
    P->maxk = 0;
    P->surf_normals = d_normals;
    P->surf_count = d_normals ? n_count : 0;
    P->surf_spacing = n_spacing;
    P->surf_spacings = d_normals ? d_n_spacings : nullptr;
    P->surf_pending = false;
    return DCPSE_OK;
}

int dcpse_plan_info(dcpse_plan_t* P, int64_t* n, int64_t* nnz, int* n_terms, int* n_outputs, int* max_neighbors) {
    if (int rc = check_plan(P)) return rc;
    if (n) *n = P->n;
    if (nnz) *nnz = P->nnz;
    if (n_terms) *n_terms = P->nterms;
    if (n_outputs) *n_outputs = P->nout;
    if (max_neighbors) *max_neighbors = P->maxk;
    return DCPSE_OK;
}

int dcpse_term_basis(dcpse_plan_t* P, int term, unsigned* exps, int cap, int* n) {
    if (int rc = check_plan(P)) return rc;
    if (term < 0 || term >= P->nterms) return fail(DCPSE_ERR_ARG, "term out of range");
    const auto& B = P->gbasis[P->term_group[term]];
    if (n) *n = (int)B.size();
    if ((int)B.size() > cap) return fail(DCPSE_ERR_CAPACITY, "cap too small for the basis");
    if (exps)
        for (size_t i = 0; i < B.size(); ++i)
            for (int d = 0; d < P->dim; ++d) exps[i * P->dim + d] = B[i].e[d];
    return DCPSE_OK;
}

int dcpse_build_neighbors(dcpse_plan_t* P, const double* d_pos, int64_t n, double rcut, const double* d_rcut_pp) {
    if (int rc = check_plan(P)) return rc;
    if (n < 0 || (n > 0 && !d_pos)) return fail(DCPSE_ERR_ARG, "bad particle array");
    if (n >= (int64_t)INT32_MAX) return fail(DCPSE_ERR_CAPACITY, "at most 2^31-1 particles");
    if (!d_rcut_pp && !(rcut > 0.0)) return fail(DCPSE_ERR_ARG, "rcut must be > 0");
    cudaStream_t s = P->stream;
    const int dim = P->dim;
    P->free_assembly();
    P->free_transpose();
    dfree(P->rowptr);
    dfree(P->cell_order);
    P->list_version++;
    dfree(P->cols);
    P->n = n;
    P->nnz = 0;
    P->maxk = 0;
    DCPSE_CK(dalloc(&P->rowptr, (size_t)n + 1));
    if (n == 0) {
        DCPSE_CK(cudaMemsetAsync(P->rowptr, 0, sizeof(int64_t), s));
        DCPSE_CK(dalloc(&P->cols, kPad));
        return DCPSE_OK;
    }
    // the support set: the domain set itself, a second set, or (surface
    // operators) either of them extended along the normals
    const double* ps = P->two_set() ? P->sup_pos : d_pos;
    int64_t ns = P->two_set() ? P->n_sup : n;
    P->surf_pending = false;
    if (P->surface()) {
        dfree(P->surf_ext);
        const int64_t next = ns * (1 + 2 * (int64_t)P->surf_count);
        DCPSE_CK(dalloc(&P->surf_ext, (size_t)std::max<int64_t>(next, 1) * dim));
        DCPSE_CK(surface_extend(dim, ps, P->surf_normals, ns, P->surf_count, P->surf_spacing, P->surf_spacings,
                                P->surf_ext, s));
        P->surf_nb = ns;
        ps = P->surf_ext;
        ns = next;
    }
    if (ns >= (int64_t)INT32_MAX) return fail(DCPSE_ERR_CAPACITY, "at most 2^31-1 support particles");
    const bool other_support = P->two_set() || P->surface();
    unsigned long long* mm = nullptr;
    DCPSE_CK(dalloc(&mm, 2 * kMaxDim));
    double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    if (P->has_box) {
        for (int d = 0; d < dim; ++d) {
            lo[d] = P->lo[d];
            hi[d] = P->hi[d];
        }
    } else {
        cudaError_t e = bounding_box(dim, d_pos, n, other_support ? ps : nullptr, other_support ? ns : 0, lo, hi, mm, s);
        if (e != cudaSuccess) {
            dfree(mm);
            return fail(DCPSE_ERR_CUDA, std::string("bounding box: ") + cudaGetErrorString(e));
        }
        for (int d = 0; d < dim; ++d) {
            P->lo[d] = lo[d];
            P->hi[d] = hi[d];
            P->per[d] = 0;
            if (!std::isfinite(lo[d]) || !std::isfinite(hi[d])) {
                dfree(mm);
                return fail(DCPSE_ERR_ARG, "non-finite particle positions");
            }
        }
    }
    double rmax = rcut;
    if (d_rcut_pp) {
        double rlo[3], rhi[3];
        cudaError_t e = bounding_box(1, d_rcut_pp, n, nullptr, 0, rlo, rhi, mm, s);
        if (e != cudaSuccess) {
            dfree(mm);
            return fail(DCPSE_ERR_CUDA, std::string("rcut range: ") + cudaGetErrorString(e));
        }
        if (!(rlo[0] > 0.0) || !std::isfinite(rhi[0])) {
            dfree(mm);
            return fail(DCPSE_ERR_ARG, "per-particle radii must be finite and > 0");
        }
        rmax = std::max(rcut > 0 ? rcut : 0.0, rhi[0]);
    }
    dfree(mm);
    // the cell list holds the support set; total cells bounded by ~4 n
    const double cap = std::max(4.0 * (double)std::max(n, ns), 1024.0);
    auto make_grid = [&](double cmin) {
        CellGrid g{};
        for (int it = 0; it < 64; ++it) {
            double total = 1.0;
            for (int d = 0; d < kMaxDim; ++d) {
                if (d < dim) {
                    double L = hi[d] - lo[d];
                    double m = (L > 0.0) ? std::floor(L / cmin) : 1.0;
                    if (!(m >= 1.0)) m = 1.0;
                    g.nc[d] = (int)std::min(m, 1.0e6);
                    g.cs[d] = (L > 0.0) ? L / (double)g.nc[d] : 1.0;
                    g.lo[d] = lo[d];
                } else {
                    g.nc[d] = 1;
                    g.cs[d] = 1.0;
                    g.lo[d] = 0.0;
                }
                total *= g.nc[d];
            }
            if (total <= cap) break;
            cmin *= 1.25;
        }
        return g;
    };
    // cells no smaller than half the largest radius, +-2 stencil (packed
    // rows), when every periodic axis then has at least five cells; else
    // cells no smaller than the largest radius and a +-1 stencil
    CellGrid cg = make_grid(0.5 * rmax * (1.0 + 1e-9));
    int packed = 1;
    for (int d = 0; d < dim; ++d)
        if (P->per[d] && cg.nc[d] < 5) packed = 0;
    if (!packed) cg = make_grid(rmax * (1.0 + 1e-9));
    const int64_t ncell = (int64_t)cg.nc[0] * cg.nc[1] * cg.nc[2];
    int32_t *cell = nullptr, *ccount = nullptr, *cidx = nullptr, *counts = nullptr, *tmp = nullptr;
    int64_t *cstart = nullptr, *fill = nullptr, *scan_tmp = nullptr;
    double* spos = nullptr;
    float4* srel = nullptr;
    int* maxk = nullptr;
    auto cleanup = [&]() {
        dfree(srel);
        dfree(cell);
        dfree(ccount);
        dfree(cidx);
        dfree(counts);
        dfree(tmp);
        dfree(cstart);
        dfree(fill);
        dfree(scan_tmp);
        dfree(spos);
        dfree(maxk);
    };
    cudaError_t e = cudaSuccess;
    if (e == cudaSuccess) e = dalloc(&cell, ns);
    if (e == cudaSuccess) e = dalloc(&ccount, ncell);
    if (e == cudaSuccess) e = dalloc(&cidx, ns);
    if (e == cudaSuccess) e = dalloc(&counts, n);
    if (e == cudaSuccess) e = dalloc(&cstart, ncell + 1);
    if (e == cudaSuccess) e = dalloc(&fill, ncell);
    if (e == cudaSuccess) e = dalloc(&scan_tmp, scan_tmp_elems(std::max<int64_t>(ncell, n)));
    if (e == cudaSuccess) e = dalloc(&spos, (size_t)ns * dim);
    if (e == cudaSuccess) e = dalloc(&srel, (size_t)std::max<int64_t>(ns, 1));
    if (e == cudaSuccess) e = dalloc(&maxk, 1);
    if (e == cudaSuccess) e = cudaMemsetAsync(maxk, 0, sizeof(int), s);
    P->tstart(DCPSE_K_NEIGHBORS);
    if (e == cudaSuccess) e = build_cells(dim, ps, ns, cg, cell, ccount, cstart, fill, cidx, spos, srel, scan_tmp, s);
    NbrArgs a{};
    a.dim = dim;
    a.pd = d_pos;
    a.n_dom = n;
    a.spos = spos;
    a.cidx = cidx;
    a.cstart = cstart;
    a.cells = cg;
    a.geom = plan_geom(P);
    a.rcut = rcut;
    a.rcut_pp = d_rcut_pp;
    a.self_skip = P->two_set() ? 0 : P->self_skip;
    a.srel = srel;
    // FP32 classification margin 2^-14 S^2, S = 3 x the largest cell side;
    // a periodic axis with fewer than three cells lists a cell under several
    // images, which only the FP64 test tells apart
    {
        double S = 0.0;
        for (int d = 0; d < dim; ++d) S = std::max(S, 3.0 * cg.cs[d]);
        a.band = std::ldexp(S * S, -14);
        for (int d = 0; d < 3; ++d) a.csf[d] = d < dim ? (float)cg.cs[d] : 0.f;
        a.packed = packed;
        a.fast = 1;
        for (int d = 0; d < dim; ++d)
            if (P->per[d] && cg.nc[d] < 3) a.fast = 0;
    }
    if (e == cudaSuccess) e = count_neighbors(a, counts, maxk, s);
    if (e == cudaSuccess) e = exclusive_scan_i32(counts, n, P->rowptr, scan_tmp, s);
    int64_t nnz = 0;
    int hk = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&nnz, P->rowptr + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hk, maxk, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = dalloc(&tmp, nnz);
    if (e == cudaSuccess) e = dalloc(&P->cols, nnz + kPad);
    if (e == cudaSuccess) e = fill_neighbors(a, P->rowptr, tmp, P->cols, hk, s);
    P->tstop(DCPSE_K_NEIGHBORS);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e == cudaSuccess && !other_support) {
        // the particles' renumbering order (one set; P->reorder_order): the
        // apply's sliced layout may renumber rows and columns by it (the
        // cells' own order, if the order's work space cannot be had)
        int32_t *key = nullptr, *zord = nullptr;
        int64_t* ztmp = nullptr;
        cudaError_t ez = dalloc(&key, (size_t)std::max<int64_t>(ns, 1));
        if (ez == cudaSuccess) ez = dalloc(&zord, (size_t)std::max<int64_t>(ns, 1));
        if (ez == cudaSuccess) ez = dalloc(&ztmp, (size_t)order_tmp_elems(dim, ns, cg, P->reorder_order));
        if (ez == cudaSuccess) ez = particle_order(dim, ps, ns, cg, P->reorder_order, key, ztmp, zord, s);
        if (ez == cudaSuccess) ez = cudaStreamSynchronize(s);
        dfree(key);
        dfree(ztmp);
        if (ez == cudaSuccess) {
            P->cell_order = zord;
        } else {
            dfree(zord);
            cudaGetLastError();
            P->cell_order = cidx;
            cidx = nullptr;
        }
    }
    cleanup();
    if (e != cudaSuccess) return fail(DCPSE_ERR_CUDA, std::string("neighbour build: ") + cudaGetErrorString(e));
    P->nnz = nnz;
    P->maxk = hk;
    P->surf_pending = P->surface();
    return DCPSE_OK;
}

int dcpse_set_neighbors(dcpse_plan_t* P, int64_t n, int64_t nnz, const int64_t* d_rowptr, const int32_t* d_cols) {
    if (int rc = check_plan(P)) return rc;
    if (P->surface()) return fail(DCPSE_ERR_STATE, "surface operators build their own lists (dcpse_build_neighbors)");
    if (n < 0 || nnz < 0 || !d_rowptr || (nnz > 0 && !d_cols)) return fail(DCPSE_ERR_ARG, "bad CSR arrays");
    cudaStream_t s = P->stream;
    P->free_assembly();
    P->free_transpose();
    dfree(P->rowptr);
    dfree(P->cell_order);
    P->list_version++;
    dfree(P->cols);
    P->n = n;
    P->nnz = nnz;
    DCPSE_CK(dalloc(&P->rowptr, (size_t)n + 1));
    DCPSE_CK(dalloc(&P->cols, nnz + kPad));
    DCPSE_CK(cudaMemcpyAsync(P->rowptr, d_rowptr, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToDevice, s));
    if (nnz > 0) DCPSE_CK(cudaMemcpyAsync(P->cols, d_cols, sizeof(int32_t) * nnz, cudaMemcpyDeviceToDevice, s));
    {
        unsigned long long* bad = nullptr;
        DCPSE_CK(dalloc(&bad, 1));
        DCPSE_CK(cudaMemsetAsync(bad, 0, sizeof(unsigned long long), s));
        int64_t work = std::max<int64_t>(n, nnz);
        csr_check_kernel<<<std::max(1, (int)std::min<int64_t>(num_sms() * 8, (work + 255) / 256)), 256, 0, s>>>(
            P->rowptr, P->cols, n, nnz, P->two_set() ? P->n_sup : n, bad);
        unsigned long long hb = 0;
        cudaError_t e = cudaMemcpyAsync(&hb, bad, sizeof hb, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        dfree(bad);
        DCPSE_CK(e);
        if (hb != 0) {
            dfree(P->rowptr);
            P->list_version++;
            dfree(P->cols);
            P->n = -1;
            P->nnz = 0;
            return fail(DCPSE_ERR_ARG, "invalid CSR neighbour list (row offsets or column indices)");
        }
    }
    int* mk = nullptr;
    DCPSE_CK(dalloc(&mk, 1));
    DCPSE_CK(cudaMemsetAsync(mk, 0, sizeof(int), s));
    if (n > 0) row_max_kernel<<<std::max(1, std::min(num_sms() * 4, (int)((n + 255) / 256))), 256, 0, s>>>(P->rowptr, n, mk);
    int hk = 0;
    DCPSE_CK(cudaMemcpyAsync(&hk, mk, sizeof(int), cudaMemcpyDeviceToHost, s));
    DCPSE_CK(cudaStreamSynchronize(s));
    dfree(mk);
    P->maxk = hk;
    return DCPSE_OK;
}

int dcpse_neighbors_ptr(dcpse_plan_t* P, const int64_t** d_rowptr, const int32_t** d_cols) {
    if (int rc = check_plan(P)) return rc;
    if (P->n < 0) return fail(DCPSE_ERR_STATE, "no neighbour list");
    if (d_rowptr) *d_rowptr = P->rowptr;
    if (d_cols) *d_cols = P->cols;
    return DCPSE_OK;
}

namespace {
int ensure_sell(dcpse_plan_t* P);
int ensure_sell64(dcpse_plan_t* P);
}  // namespace

int dcpse_assemble(dcpse_plan_t* P, const double* d_pos, const double* d_eps_fixed, int flags) {
    if (int rc = check_plan(P)) return rc;
    if (P->n < 0) return fail(DCPSE_ERR_STATE, "build or set the neighbour list first");
    if (P->n > 0 && !d_pos) return fail(DCPSE_ERR_ARG, "NULL positions");
    if (!(flags & (DCPSE_STORE_TERMS_F64 | DCPSE_STORE_OUT_F64 | DCPSE_STORE_OUT_F32)))
        return fail(DCPSE_ERR_ARG, "nothing to store");
    if ((flags & DCPSE_ASSEMBLE_FAST) && (flags & DCPSE_STORE_TERMS_F64))
        return fail(DCPSE_ERR_ARG, "per-term kernels need the reference (non-fast) assembly");
    if ((flags & (DCPSE_STORE_OUT_F32_RESID | DCPSE_STORE_OUT_F32_CORR)) && !(flags & DCPSE_STORE_OUT_F32))
        return fail(DCPSE_ERR_ARG, "residuals need DCPSE_STORE_OUT_F32");
    if (P->surface() && !P->surf_pending)
        return fail(DCPSE_ERR_STATE, "surface operators assemble once per neighbour build (build it again)");
    // surface operators accumulate FP64 values; FP32 weights follow from them
    const int user_flags = flags;
    if (P->surface()) {
        if (flags & DCPSE_STORE_OUT_F32) flags |= DCPSE_STORE_OUT_F64;
        flags &= ~(DCPSE_STORE_OUT_F32 | DCPSE_STORE_OUT_F32_RESID | DCPSE_STORE_OUT_F32_CORR);
    }
    cudaStream_t s = P->stream;
    const int64_t n = P->n, nnz = P->nnz;
    const int ng = P->htab->ngroups;
    // (re)allocate what this assembly stores
    if (!P->eps) DCPSE_CK(dalloc(&P->eps, n));
    if (!P->status) DCPSE_CK(dalloc(&P->status, n));
    if (!P->eip_group) DCPSE_CK(dalloc(&P->eip_group, (size_t)ng * n));
    if ((flags & DCPSE_STORE_TERMS_F64) && !P->k_term) DCPSE_CK(dalloc(&P->k_term, (size_t)P->nterms * nnz));
    if (!(flags & DCPSE_STORE_TERMS_F64)) dfree(P->k_term);
    if ((flags & DCPSE_STORE_OUT_F64) && !P->w64) DCPSE_CK(dalloc(&P->w64, (size_t)P->nout * nnz));
    if (!(flags & DCPSE_STORE_OUT_F64)) dfree(P->w64);
    P->free_sell();  // the FP32 weights are rewritten
    // so are the field VJP's row sums and transposed weights
    dfree(P->rowsum);
    P->rowsum_prec = -1;
    P->free_vsell_weights();
    if ((flags & DCPSE_STORE_OUT_F32) && !P->w32) DCPSE_CK(dalloc(&P->w32, (size_t)P->nout * nnz + kPad));
    if (!(flags & DCPSE_STORE_OUT_F32)) dfree(P->w32);
    if ((flags & DCPSE_STORE_OUT_F32_RESID) && !P->r16)
        DCPSE_CK(cudaMalloc(&P->r16, ((size_t)P->nout * nnz + kPad) * 2));
    if (!(flags & DCPSE_STORE_OUT_F32_RESID) && P->r16) {
        cudaFree(P->r16);
        P->r16 = nullptr;
    }
    if ((flags & DCPSE_STORE_OUT_F32_CORR) && !P->r32) DCPSE_CK(dalloc(&P->r32, (size_t)P->nout * nnz + kPad));
    if (!(flags & DCPSE_STORE_OUT_F32_CORR)) dfree(P->r32);
    AsmArgs a{};
    a.tab = P->dtab;
    a.dim = P->dim;
    a.n = n;
    a.pos = d_pos;
    a.spos = P->surface() ? P->surf_ext : (P->two_set() ? P->sup_pos : d_pos);
    a.rowptr = P->rowptr;
    a.cols = P->cols;
    a.geom = plan_geom(P);
    a.h_over_eps = P->hoe;
    a.eps_fixed = d_eps_fixed;
    a.flags = flags;
    a.eps = P->eps;
    a.status = P->status;
    a.eip_group = P->eip_group;
    a.k_term = P->k_term;
    a.w64 = P->w64;
    a.w32 = P->w32;
    a.r16 = P->r16;
    a.r32 = P->r32;
    a.nnz = nnz;
    a.warps = P->asm_warps;
    a.qr_lanes = P->asm_qr_lanes;
    a.maxk = P->maxk;
    a.err = P->d_err;
    a.order = nullptr;
    if (n > 0) {
        // batches of at most kAsmScratchBytes of scratch (Gram entries and
        // coefficients of the particles in flight)
        const int64_t per = assembly_scratch_bytes(*P->htab, flags, P->maxk);
        const int64_t nb = std::min<int64_t>(n, std::max<int64_t>(4096, kAsmScratchBytes / per));
        const int64_t bytes = nb * per + 16;
        if (P->asm_scratch_bytes < bytes) {
            dfree(P->asm_scratch);
            P->asm_scratch_bytes = 0;
            DCPSE_CK(dalloc(&P->asm_scratch, (size_t)(bytes + 7) / 8));
            P->asm_scratch_bytes = bytes;
        }
        a.scratch = P->asm_scratch;
        const int64_t qb = assembly_qr_ws_bytes(*P->htab, flags);
        if (qb > 0 && P->qr_ws_bytes < qb) {
            dfree(P->qr_ws);
            P->qr_ws_bytes = 0;
            DCPSE_CK(dalloc(&P->qr_ws, (size_t)(qb + 7) / 8));
            P->qr_ws_bytes = qb;
        }
        a.qws = qb > 0 ? P->qr_ws : nullptr;
        a.scratch_particles = nb;
    }
    if (P->asm_bin_width > 0 && n > 0) {
        if (!P->korder || P->korder_width != P->asm_bin_width) {
            if (!P->korder) DCPSE_CK(dalloc(&P->korder, n));
            const int64_t nb = P->maxk / P->asm_bin_width + 1;
            int32_t* hist = nullptr;
            int64_t* tmp = nullptr;
            DCPSE_CK(dalloc(&hist, nb));
            DCPSE_CK(dalloc(&tmp, binning_tmp_elems(n, P->maxk, P->asm_bin_width)));
            cudaError_t eb = bin_by_count(P->rowptr, n, P->maxk, P->asm_bin_width, P->korder, hist, tmp, s);
            if (eb == cudaSuccess) eb = cudaStreamSynchronize(s);
            dfree(hist);
            dfree(tmp);
            DCPSE_CK(eb);
            P->korder_width = P->asm_bin_width;
        }
        a.order = P->korder;
    }
    P->asm_tc = assembly_uses_tc(*P->htab, flags, P->maxk);
    P->tstart(DCPSE_K_ASSEMBLE);
    cudaError_t e = assemble(a, *P->htab, s);
    if (e == cudaErrorInvalidConfiguration)
        return fail(DCPSE_ERR_CAPACITY, "assembly: the QR work space of this lane grouping exceeds shared memory");
    if (e != cudaSuccess) return fail(DCPSE_ERR_CUDA, std::string("assembly: ") + cudaGetErrorString(e));
    // the FP32 weights on the sliced ELL layout of the default apply are
    // part of the assembly (surface operators: after the accumulation)
    if ((flags & DCPSE_STORE_OUT_F32) && !P->surface())
        if (int rc = ensure_sell(P)) return rc;
    P->tstop(DCPSE_K_ASSEMBLE);
    if (P->surface()) {
        if (int rc = surface_finish(P, user_flags)) return rc;
        flags = user_flags;
    }
    P->assembled = true;
    P->flags = flags;
    unsigned long long init[2] = {0ull, ~0ull};
    DCPSE_CK(cudaMemcpyAsync(P->summary, init, sizeof init, cudaMemcpyHostToDevice, s));
    if (n > 0)
        status_summary_kernel<<<std::max(1, std::min(num_sms() * 4, (int)((n + 255) / 256))), 256, 0, s>>>(
            P->status, n, P->summary);
    DCPSE_CK(cudaGetLastError());
    if (flags & DCPSE_ASSEMBLE_ASYNC) return DCPSE_OK;
    int64_t nb = 0, fb = -1;
    int fc = 0;
    int rc = dcpse_particle_status(P, &nb, &fb, &fc);
    if (rc != DCPSE_OK) return rc;
    if (nb > 0) {
        char buf[160];
        std::snprintf(buf, sizeof buf, "%lld particle(s) could not be assembled; first %lld (status %d)",
                      (long long)nb, (long long)fb, fc);
        return fail(DCPSE_ERR_PARTICLES, buf);
    }
    return DCPSE_OK;
}

int dcpse_particle_status(dcpse_plan_t* P, int64_t* n_bad, int64_t* first_bad, int* first_code) {
    if (int rc = check_plan(P)) return rc;
    if (!P->assembled) return fail(DCPSE_ERR_STATE, "not assembled");
    unsigned long long h[2];
    DCPSE_CK(cudaMemcpyAsync(h, P->summary, sizeof h, cudaMemcpyDeviceToHost, P->stream));
    DCPSE_CK(cudaStreamSynchronize(P->stream));
    int code = 0;
    if (h[0] > 0)
        DCPSE_CK(cudaMemcpy(&code, P->status + h[1], sizeof(int), cudaMemcpyDeviceToHost));
    if (n_bad) *n_bad = (int64_t)h[0];
    if (first_bad) *first_bad = h[0] > 0 ? (int64_t)h[1] : -1;
    if (first_code) *first_code = code;
    return DCPSE_OK;
}

int dcpse_eps_ptr(dcpse_plan_t* P, const double** d_eps, const int32_t** d_status) {
    if (int rc = check_plan(P)) return rc;
    if (!P->assembled) return fail(DCPSE_ERR_STATE, "not assembled");
    if (d_eps) *d_eps = P->eps;
    if (d_status) *d_status = P->status;
    return DCPSE_OK;
}

int dcpse_term_kernels_ptr(dcpse_plan_t* P, int term, const double** d_kernels, const double** d_eps_inv_pow) {
    if (int rc = check_plan(P)) return rc;
    if (!P->assembled) return fail(DCPSE_ERR_STATE, "not assembled");
    if (term < 0 || term >= P->nterms) return fail(DCPSE_ERR_ARG, "term out of range");
    if (d_kernels) *d_kernels = P->k_term ? P->k_term + (size_t)term * P->nnz : nullptr;
    if (d_eps_inv_pow) *d_eps_inv_pow = P->eip_group + (size_t)P->term_group[term] * P->n;
    return DCPSE_OK;
}

int dcpse_output_weights_ptr(dcpse_plan_t* P, int output, const double** d_w64, const float** d_w32) {
    if (int rc = check_plan(P)) return rc;
    if (!P->assembled) return fail(DCPSE_ERR_STATE, "not assembled");
    if (output < 0 || output >= P->nout) return fail(DCPSE_ERR_ARG, "output out of range");
    if (d_w64) *d_w64 = P->w64 ? P->w64 + (size_t)output * P->nnz : nullptr;
    if (d_w32) *d_w32 = P->w32 ? P->w32 + (size_t)output * P->nnz : nullptr;
    return DCPSE_OK;
}

int dcpse_set_term_kernels(dcpse_plan_t* P, int term, const double* d_kernels, const double* d_eps,
                           const double* d_eps_inv_pow) {
    if (int rc = check_plan(P)) return rc;
    if (P->n < 0) return fail(DCPSE_ERR_STATE, "set the neighbour list first");
    if (term < 0 || term >= P->nterms) return fail(DCPSE_ERR_ARG, "term out of range");
    if ((P->nnz > 0 && !d_kernels) || (P->n > 0 && (!d_eps || !d_eps_inv_pow)))
        return fail(DCPSE_ERR_ARG, "NULL array");
    const int64_t n = P->n, nnz = P->nnz;
    if (!P->assembled) {
        // fresh plan (support_options::LOAD): kernels of every term start at zero
        P->free_assembly();
        DCPSE_CK(dalloc(&P->eps, n));
        DCPSE_CK(dalloc(&P->status, n));
        DCPSE_CK(dalloc(&P->eip_group, (size_t)P->htab->ngroups * n));
        DCPSE_CK(dalloc(&P->k_term, (size_t)P->nterms * nnz));
        DCPSE_CK(cudaMemsetAsync(P->status, 0, sizeof(int32_t) * n, P->stream));
        DCPSE_CK(cudaMemsetAsync(P->k_term, 0, sizeof(double) * P->nterms * nnz, P->stream));
        unsigned long long init[2] = {0ull, ~0ull};
        DCPSE_CK(cudaMemcpyAsync(P->summary, init, sizeof init, cudaMemcpyHostToDevice, P->stream));
        P->assembled = true;
        P->flags = DCPSE_STORE_TERMS_F64;
    }
    if (!P->k_term) return fail(DCPSE_ERR_STATE, "plan was assembled without per-term kernels");
    // summed output weights of an earlier assembly no longer match: drop
    // them (the batched applies then ask for a new assembly)
    P->free_sell();
    dfree(P->w64);
    dfree(P->w32);
    if (P->r16) cudaFree(P->r16);
    P->r16 = nullptr;
    P->flags &= ~(DCPSE_STORE_OUT_F64 | DCPSE_STORE_OUT_F32 | DCPSE_STORE_OUT_F32_RESID);
    dfree(P->rowsum);
    P->rowsum_prec = -1;
    P->free_vsell_weights();
    cudaStream_t s = P->stream;
    if (nnz > 0)
        DCPSE_CK(cudaMemcpyAsync(P->k_term + (size_t)term * nnz, d_kernels, sizeof(double) * nnz,
                                 cudaMemcpyDefault, s));
    if (n > 0) {
        DCPSE_CK(cudaMemcpyAsync(P->eps, d_eps, sizeof(double) * n, cudaMemcpyDefault, s));
        DCPSE_CK(cudaMemcpyAsync(P->eip_group + (size_t)P->term_group[term] * n, d_eps_inv_pow, sizeof(double) * n,
                                 cudaMemcpyDefault, s));
    }
    DCPSE_CK(cudaStreamSynchronize(s));
    return DCPSE_OK;
}

namespace {
int ensure_transpose(dcpse_plan_t* P) {
    if (P->t_row) return DCPSE_OK;
    cudaStream_t s = P->stream;
    const int64_t n = P->n, nnz = P->nnz;
    int32_t *cnt = nullptr, *src_tmp = nullptr;
    int64_t *fill = nullptr, *idx_tmp = nullptr, *scan_tmp = nullptr;
    cudaError_t e = dalloc(&P->t_row, (size_t)n + 1);
    if (e == cudaSuccess) e = dalloc(&P->t_src, nnz);
    if (e == cudaSuccess) e = dalloc(&P->t_idx, nnz);
    if (e == cudaSuccess) e = dalloc(&cnt, n);
    if (e == cudaSuccess) e = dalloc(&fill, n);
    if (e == cudaSuccess) e = dalloc(&src_tmp, nnz);
    if (e == cudaSuccess) e = dalloc(&idx_tmp, nnz);
    if (e == cudaSuccess) e = dalloc(&scan_tmp, scan_tmp_elems(n));
    if (e == cudaSuccess && n == 0) e = cudaMemsetAsync(P->t_row, 0, sizeof(int64_t), s);
    if (e == cudaSuccess)
        e = build_transpose(P->rowptr, P->cols, n, nnz, cnt, P->t_row, fill, src_tmp, idx_tmp, P->t_src, P->t_idx,
                            scan_tmp, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    dfree(cnt);
    dfree(fill);
    dfree(src_tmp);
    dfree(idx_tmp);
    dfree(scan_tmp);
    if (e != cudaSuccess) {
        P->free_transpose();
        return fail(DCPSE_ERR_CUDA, std::string("transposed list: ") + cudaGetErrorString(e));
    }
    return DCPSE_OK;
}
}  // namespace

namespace {
// The field VJP's sliced layout of the transposed list and, for precision,
// the transposed weights of every output on it; without room the CSR
// kernel serves (*ready false).
int ensure_vjp_sell(dcpse_plan_t* P, int precision, bool* ready) {
    *ready = false;
    if (P->n == 0 || P->vsell_no_room) return DCPSE_OK;
    cudaStream_t st = P->stream;
    cudaError_t e = cudaSuccess;
    if (!P->vsell_row) {
        const int64_t ns = sell_slices(P->n);
        int32_t* slen = nullptr;
        int64_t* tmp = nullptr;
        int64_t total = 0;
        e = dalloc(&P->vsell_row, (size_t)ns * 32);
        if (e == cudaSuccess) e = dalloc(&P->vsell_off, (size_t)ns + 1);
        if (e == cudaSuccess) e = dalloc(&slen, (size_t)ns);
        if (e == cudaSuccess) e = dalloc(&tmp, (size_t)scan_tmp_elems(ns));
        if (e == cudaSuccess) e = sell_order(P->t_row, P->n, P->vsell_row, slen, P->vsell_off, tmp, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&total, P->vsell_off + ns, sizeof total, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        dfree(slen);
        dfree(tmp);
        if (e == cudaSuccess) e = dalloc(&P->vsell_cols, (size_t)total + kPad);
        // the columns: the source particles, padding on the row itself
        if (e == cudaSuccess)
            e = sell_fill(P->t_row, P->t_src, nullptr, nullptr, P->nnz, P->nout, P->n, 1, P->vsell_row, P->vsell_off,
                          total, P->vsell_cols, nullptr, nullptr, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e == cudaSuccess) P->vsell_total = total;
    }
    const bool f64 = precision == DCPSE_F64;
    double*& lw = f64 ? P->vsell_w64 : P->vsell_w32;
    if (e == cudaSuccess && !lw) {
        // transposed weights of every output (CSR order, as doubles: FP32
        // weights widened once here instead of at every use), then on the
        // layout
        double* wt = nullptr;
        e = dalloc(&wt, (size_t)P->nout * P->nnz + kPad);
        if (e == cudaSuccess)
            e = transpose_outputs(P->t_idx, P->nnz, P->nout, f64 ? P->w64 : nullptr, f64 ? nullptr : P->w32, P->nnz,
                                  wt, st);
        if (e == cudaSuccess) e = dalloc(&lw, (size_t)P->nout * P->vsell_total + kPad);
        if (e == cudaSuccess)
            e = sell_fill64(P->t_row, wt, P->nnz, P->nout, P->n, P->vsell_row, P->vsell_off, P->vsell_total, lw, st,
                            nullptr);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        dfree(wt);
    }
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        P->free_vsell();
        P->vsell_no_room = true;
        return DCPSE_OK;
    }
    if (e != cudaSuccess) {
        P->free_vsell();
        return fail(DCPSE_ERR_CUDA, std::string("field VJP layout: ") + cudaGetErrorString(e));
    }
    *ready = true;
    return DCPSE_OK;
}
}  // namespace

int dcpse_vjp_field(dcpse_plan_t* P, const double* d_g, double* d_out, int precision) {
    if (int rc = check_plan(P)) return rc;
    if (int rc = check_single_set(P)) return rc;
    if (!P->assembled) return fail(DCPSE_ERR_STATE, "not assembled");
    if (P->n > 0 && (!d_g || !d_out)) return fail(DCPSE_ERR_ARG, "NULL array");
    const double* w64 = nullptr;
    const float* w32 = nullptr;
    if (precision == DCPSE_F64) {
        if (!P->w64) return fail(DCPSE_ERR_STATE, "FP64 output weights not stored");
        w64 = P->w64;
    } else if (precision == DCPSE_F32) {
        if (!P->w32) return fail(DCPSE_ERR_STATE, "FP32 weights not stored");
        w32 = P->w32;
    } else {
        return fail(DCPSE_ERR_ARG, "precision must be DCPSE_F64 or DCPSE_F32");
    }
    if (int rc = ensure_transpose(P)) return rc;
    if (P->rowsum_prec != precision) {
        if (!P->rowsum) DCPSE_CK(dalloc(&P->rowsum, (size_t)P->nout * P->n));
        DCPSE_CK(row_sums(P->rowptr, P->n, P->nout, w64, w32, P->nnz, P->rowsum, P->stream));
        P->rowsum_prec = precision;
    }
    // the sliced kernel unless a CSR schedule was asked for
    const int mode = P->apply_mode & 15;
    if (mode == 0 || mode == 4) {
        bool ready = false;
        if (int rc = ensure_vjp_sell(P, precision, &ready)) return rc;
        if (ready) {
            VjpSellArgs a{};
            a.n = P->n;
            a.nwin = (P->n + 255) / 256;
            a.srow = P->vsell_row;
            a.off = P->vsell_off;
            a.cols = P->vsell_cols;
            a.w = w64 ? P->vsell_w64 : P->vsell_w32;
            a.total = P->vsell_total;
            a.rs = P->rowsum;
            a.g = d_g;
            a.out = d_out;
            DCPSE_CK(vjp_field_sell(a, P->nout, P->stream));
            return DCPSE_OK;
        }
    }
    DCPSE_CK(vjp_field(P->t_row, P->t_src, P->t_idx, P->n, P->nout, w64, w32, P->nnz, P->rowsum, d_g, d_out,
                       P->stream));
    return DCPSE_OK;
}

int dcpse_vjp_positions(dcpse_plan_t* P, const double* d_pos, const double* d_eps_fixed, const double* d_f,
                        const double* d_g, double* d_grad) {
    if (int rc = check_plan(P)) return rc;
    if (int rc = check_single_set(P)) return rc;
    if (P->n < 0) return fail(DCPSE_ERR_STATE, "no neighbour list");
    if (P->n > 0 && (!d_pos || !d_f || !d_g || !d_grad)) return fail(DCPSE_ERR_ARG, "NULL array");
    for (int g = 0; g < P->htab->ngroups; ++g)
        if (P->htab->gn[g] > kMaxBasisSmall)
            return fail(DCPSE_ERR_CAPACITY, "position VJP: bases of at most 35 functions");
    if (int rc = ensure_transpose(P)) return rc;
    if (!P->gentry) DCPSE_CK(dalloc(&P->gentry, (size_t)P->nnz * P->dim));
    VjpArgs a{};
    a.tab = P->dtab;
    a.n = P->n;
    a.pos = d_pos;
    a.rowptr = P->rowptr;
    a.cols = P->cols;
    a.geom = plan_geom(P);
    a.h_over_eps = P->hoe;
    a.eps_fixed = d_eps_fixed;
    a.f = d_f;
    a.gbar = d_g;
    a.gentry = P->gentry;
    DCPSE_CK(vjp_positions(a, *P->htab, P->t_row, P->t_idx, d_grad, P->stream));
    return DCPSE_OK;
}

// RK4 stage kernels: lanes per row for 16 to 32 neighbour entries per lane in
// 4-deep batches (96^3 periodic cloud, 84 entries per row: 4 lanes 0.79 ms
// per step, 8 lanes 0.85 ms, 16 lanes 1.26 ms)
static int rk_lanes(const dcpse_plan_t* P) {
    if (P->apply_lanes) return P->apply_lanes;
    const double avg = P->n > 0 ? (double)P->nnz / (double)P->n : 0.0;
    int lanes = 4;
    while (lanes < 32 && avg / (2 * lanes) >= 16.0) lanes *= 2;
    return lanes;
}

// the gathered input of an RK4 stage or adjoint stage as (u, v) pairs: plan
// scratch, 16 bytes per particle
static int ensure_rk_pack(dcpse_plan_t* P) {
    if (P->rk_pack_n < P->n) {
        dfree(P->rk_pack);
        P->rk_pack_n = 0;
        // two areas of n pairs: stage input, and the fused reverse step's second kbar
        DCPSE_CK(dalloc(&P->rk_pack, (size_t)std::max<int64_t>(P->n, 1) * 4));
        P->rk_pack_n = P->n;
    }
    return DCPSE_OK;
}

int dcpse_rk4_gs_stage(dcpse_plan_t* P, int stage, int precision, const void* Yu, const void* Yv, const void* y0u,
                       const void* y0v, void* accu, void* accv, void* outu, void* outv, const double* params) {
    if (int rc = check_plan(P)) return rc;
    if (int rc = check_single_set(P)) return rc;
    if (!P->assembled) return fail(DCPSE_ERR_STATE, "not assembled");
    if (stage < 0 || stage > 3 || !params) return fail(DCPSE_ERR_ARG, "stage 0..3 and params {Du,Dv,F,k,dt}");
    if (P->n > 0 && (!Yu || !Yv || !y0u || !y0v || !accu || !accv || !outu || !outv))
        return fail(DCPSE_ERR_ARG, "NULL array");
    const int lanes = rk_lanes(P);
    if (int rc = ensure_rk_pack(P)) return rc;
    if (precision == DCPSE_F32) {
        if (!P->w32) return fail(DCPSE_ERR_STATE, "FP32 weights not stored");
        RkArgs<float> a{P->n, P->rowptr, P->cols, P->w32, (const float*)Yu, (const float*)Yv, (const float*)y0u,
                        (const float*)y0v, (float*)accu, (float*)accv, (float*)outu, (float*)outv,
                        params[0], params[1], params[2], params[3], params[4], stage, P->rk_pack,
                        nullptr, nullptr, nullptr, nullptr};
        // the sliced ELL layout of the Laplacian's weights (output 0), unless
        // a CSR schedule was asked for
        const int mode = P->apply_mode & 15;
        if (mode == 0 || mode == 4) {
            if (int rc = ensure_sell(P)) return rc;
            if (P->sell_w && !P->sell_perm) {  // the stage kernels read fields in list order
                a.srow = P->sell_row;
                a.soff = P->sell_off;
                a.scols = P->sell_cols;
                a.sw = P->sell_w;
            }
        }
        DCPSE_CK(rk_stage<float>(a, lanes, P->stream));
    } else if (precision == DCPSE_F64) {
        if (!P->w64) return fail(DCPSE_ERR_STATE, "FP64 output weights not stored");
        RkArgs<double> a{P->n, P->rowptr, P->cols, P->w64, (const double*)Yu, (const double*)Yv, (const double*)y0u,
                         (const double*)y0v, (double*)accu, (double*)accv, (double*)outu, (double*)outv,
                         params[0], params[1], params[2], params[3], params[4], stage, P->rk_pack,
                         nullptr, nullptr, nullptr, nullptr};
        DCPSE_CK(rk_stage<double>(a, lanes, P->stream));
    } else {
        return fail(DCPSE_ERR_ARG, "precision must be DCPSE_F32 or DCPSE_F64");
    }
    return DCPSE_OK;
}

int dcpse_rk4_gs_adjoint_prepare(dcpse_plan_t* P, int precision) {
    if (int rc = check_plan(P)) return rc;
    if (int rc = check_single_set(P)) return rc;
    if (!P->assembled) return fail(DCPSE_ERR_STATE, "not assembled");
    if (int rc = ensure_transpose(P)) return rc;
    if (precision == DCPSE_F32) {
        if (!P->w32) return fail(DCPSE_ERR_STATE, "FP32 weights not stored");
        if (!P->wT32) DCPSE_CK(dalloc(&P->wT32, P->nnz));
        if (!P->rs32) DCPSE_CK(dalloc(&P->rs32, P->n));
        DCPSE_CK(rk_transpose_weights<float>(P->rowptr, P->t_idx, P->n, P->nnz, P->w32, P->wT32, P->rs32, P->stream));
        // the transposed list and weights on a sliced ELL layout (the forward
        // stage's layout, for the adjoint stage): kept only if it fits
        P->free_tsell();
        if (P->n > 0) {
            const int64_t ns = sell_slices(P->n);
            int32_t* slen = nullptr;
            int64_t* tmp = nullptr;
            int64_t total = 0;
            cudaError_t e = dalloc(&P->tsell_row, (size_t)ns * 32);
            if (e == cudaSuccess) e = dalloc(&P->tsell_off, (size_t)ns + 1);
            if (e == cudaSuccess) e = dalloc(&slen, (size_t)ns);
            if (e == cudaSuccess) e = dalloc(&tmp, (size_t)scan_tmp_elems(ns));
            if (e == cudaSuccess) e = sell_order(P->t_row, P->n, P->tsell_row, slen, P->tsell_off, tmp, P->stream);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(&total, P->tsell_off + ns, sizeof total, cudaMemcpyDeviceToHost, P->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(P->stream);
            dfree(slen);
            dfree(tmp);
            if (e == cudaSuccess) e = dalloc(&P->tsell_cols, (size_t)total + kPad);
            if (e == cudaSuccess) e = dalloc(&P->tsell_w, (size_t)total + kPad);
            if (e == cudaSuccess)
                e = sell_fill(P->t_row, P->t_src, P->wT32, nullptr, P->nnz, 1, P->n, 1, P->tsell_row, P->tsell_off,
                              total, P->tsell_cols, P->tsell_w, nullptr, P->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(P->stream);
            if (e != cudaSuccess) {
                P->free_tsell();
                if (e != cudaErrorMemoryAllocation) return fail(DCPSE_ERR_CUDA, cudaGetErrorString(e));
                cudaGetLastError();  // no room: the CSR adjoint kernel serves
            }
        }
    } else if (precision == DCPSE_F64) {
        if (!P->w64) return fail(DCPSE_ERR_STATE, "FP64 output weights not stored");
        if (!P->wT64) DCPSE_CK(dalloc(&P->wT64, P->nnz));
        if (!P->rs64) DCPSE_CK(dalloc(&P->rs64, P->n));
        DCPSE_CK(rk_transpose_weights<double>(P->rowptr, P->t_idx, P->n, P->nnz, P->w64, P->wT64, P->rs64, P->stream));
    } else {
        return fail(DCPSE_ERR_ARG, "precision must be DCPSE_F32 or DCPSE_F64");
    }
    if (int rc = ensure_rk_pack(P)) return rc;
    DCPSE_CK(cudaStreamSynchronize(P->stream));
    return DCPSE_OK;
}

int dcpse_rk4_gs_adjoint_stage(dcpse_plan_t* P, int precision, const void* Yu, const void* Yv, const void* kbu,
                               const void* kbv, const void* ybu, const void* ybv, void* accu, void* accv, void* next_u,
                               void* next_v, double cy, double cY, const double* params) {
    if (int rc = check_plan(P)) return rc;
    if (!params) return fail(DCPSE_ERR_ARG, "params {Du,Dv,F,k,dt}");
    if (P->n > 0 && (!Yu || !Yv || !kbu || !kbv || !ybu || !ybv || !accu || !accv))
        return fail(DCPSE_ERR_ARG, "NULL array");
    if (P->rk_pack_n < P->n) return fail(DCPSE_ERR_STATE, "call dcpse_rk4_gs_adjoint_prepare first");
    const int lanes = rk_lanes(P);
    if (precision == DCPSE_F32) {
        if (!P->wT32) return fail(DCPSE_ERR_STATE, "call dcpse_rk4_gs_adjoint_prepare first");
        RkAdjArgs<float> a{P->n, P->t_row, P->t_src, P->wT32, P->rs32, (const float*)Yu, (const float*)Yv,
                           (const float*)kbu, (const float*)kbv, (const float*)ybu, (const float*)ybv, (float*)accu,
                           (float*)accv, (float*)next_u, (float*)next_v, cy, cY, params[0], params[1], params[2],
                           params[3], P->rk_pack, P->tsell_row, P->tsell_off, P->tsell_cols, P->tsell_w};
        const int mode = P->apply_mode & 15;
        if (!(mode == 0 || mode == 4) || !P->tsell_w) a.srow = nullptr;  // a CSR schedule was asked for
        DCPSE_CK(rk_adjoint_stage<float>(a, lanes, P->stream));
    } else if (precision == DCPSE_F64) {
        if (!P->wT64) return fail(DCPSE_ERR_STATE, "call dcpse_rk4_gs_adjoint_prepare first");
        RkAdjArgs<double> a{P->n, P->t_row, P->t_src, P->wT64, P->rs64, (const double*)Yu, (const double*)Yv,
                            (const double*)kbu, (const double*)kbv, (const double*)ybu, (const double*)ybv,
                            (double*)accu, (double*)accv, (double*)next_u, (double*)next_v, cy, cY, params[0],
                            params[1], params[2], params[3], P->rk_pack, nullptr, nullptr, nullptr, nullptr};
        DCPSE_CK(rk_adjoint_stage<double>(a, lanes, P->stream));
    } else {
        return fail(DCPSE_ERR_ARG, "precision must be DCPSE_F32 or DCPSE_F64");
    }
    return DCPSE_OK;
}

int dcpse_rk4_gs_reverse_step(dcpse_plan_t* P, int precision, const void* const* stages, void* ybu, void* ybv,
                              void* accu, void* accv, const double* params) {
    if (int rc = check_plan(P)) return rc;
    if (!params || !stages) return fail(DCPSE_ERR_ARG, "stages {Y1u,Y1v,...,Y4u,Y4v} and params {Du,Dv,F,k,dt}");
    if (P->n > 0 && (!ybu || !ybv || !accu || !accv)) return fail(DCPSE_ERR_ARG, "NULL array");
    for (int i = 0; i < 8 && P->n > 0; ++i)
        if (!stages[i]) return fail(DCPSE_ERR_ARG, "NULL stage state");
    if (P->rk_pack_n < P->n) return fail(DCPSE_ERR_STATE, "call dcpse_rk4_gs_adjoint_prepare first");
    const int lanes = rk_lanes(P);
    const double dt = params[4];
    // kbar of stages 4..1 alternate between the two pair areas; the
    // coefficients of the next kbar (RK4's weights 1/6, 1/3, 1/3, 1/6 and
    // stage offsets 1, 1/2, 1/2)
    const double cy[4] = {0.0, dt / 6.0, dt / 3.0, dt / 3.0}, cY[4] = {0.0, dt / 2.0, dt / 2.0, dt};
    auto run = [&](auto tag) -> int {
        typedef decltype(tag) T;
        typedef typename std::conditional<std::is_same<T, float>::value, float, double>::type R;
        const bool f32 = std::is_same<R, float>::value;
        const R* wT = f32 ? (const R*)(const void*)P->wT32 : (const R*)(const void*)P->wT64;
        const R* rs = f32 ? (const R*)(const void*)P->rs32 : (const R*)(const void*)P->rs64;
        if (!wT || !rs) return fail(DCPSE_ERR_STATE, "call dcpse_rk4_gs_adjoint_prepare first");
        void* area[2] = {P->rk_pack, P->rk_pack + 2 * P->rk_pack_n};
        DCPSE_CK(rk_pack_scaled<R>((const R*)ybu, (const R*)ybv, P->n, dt / 6.0, area[0], P->stream));
        for (int st = 3, cur = 0; st >= 0; --st, cur ^= 1) {
            RkAdjArgs<R> a{};
            a.n = P->n;
            a.trow = P->t_row;
            a.tsrc = P->t_src;
            a.wT = wT;
            a.rs = rs;
            a.Yu = (const R*)stages[2 * st];
            a.Yv = (const R*)stages[2 * st + 1];
            a.ybu = (const R*)ybu;
            a.ybv = (const R*)ybv;
            a.accu = (R*)accu;
            a.accv = (R*)accv;
            a.cy = cy[st];
            a.cY = cY[st];
            a.Du = params[0];
            a.Dv = params[1];
            a.F = params[2];
            a.K = params[3];
            a.pack = area[cur];
            a.kb_packed = true;
            a.pack_out = st > 0 ? area[cur ^ 1] : nullptr;
            a.acc_mode = st == 3 ? 1 : (st == 0 ? 2 : 0);
            a.yb_out_u = (R*)ybu;
            a.yb_out_v = (R*)ybv;
            const int mode = P->apply_mode & 15;
            if (f32 && (mode == 0 || mode == 4) && P->tsell_w) {
                a.srow = P->tsell_row;
                a.soff = P->tsell_off;
                a.scols = P->tsell_cols;
                a.sw = P->tsell_w;
            }
            DCPSE_CK(rk_adjoint_stage<R>(a, lanes, P->stream));
        }
        return DCPSE_OK;
    };
    if (precision == DCPSE_F32) return run(float{});
    if (precision == DCPSE_F64) return run(double{});
    return fail(DCPSE_ERR_ARG, "precision must be DCPSE_F32 or DCPSE_F64");
}

int dcpse_device_alloc(void** ptr, uint64_t bytes) {
    if (!ptr) return fail(DCPSE_ERR_ARG, "NULL pointer");
    *ptr = nullptr;
    DCPSE_CK(cudaMalloc(ptr, bytes ? bytes : 1));
    return DCPSE_OK;
}

int dcpse_device_free(void* ptr) {
    if (ptr) DCPSE_CK(cudaFree(ptr));
    return DCPSE_OK;
}

int dcpse_host_alloc(void** ptr, uint64_t bytes) {
    if (!ptr) return fail(DCPSE_ERR_ARG, "NULL pointer");
    *ptr = nullptr;
    DCPSE_CK(cudaHostAlloc(ptr, bytes ? bytes : 1, cudaHostAllocMapped | cudaHostAllocPortable));
    return DCPSE_OK;
}

int dcpse_host_free(void* ptr) {
    if (ptr) DCPSE_CK(cudaFreeHost(ptr));
    return DCPSE_OK;
}

int dcpse_copy(void* dst, const void* src, uint64_t bytes) {
    if (bytes == 0) return DCPSE_OK;
    if (!dst || !src) return fail(DCPSE_ERR_ARG, "NULL pointer");
    DCPSE_CK(cudaMemcpy(dst, src, bytes, cudaMemcpyDefault));
    return DCPSE_OK;
}

int dcpse_apply_term_f64(dcpse_plan_t* P, int term, const double* d_f, double* d_out) {
    if (int rc = check_plan(P)) return rc;
    if (int rc = check_single_set(P)) return rc;
    if (!P->assembled || !P->k_term) return fail(DCPSE_ERR_STATE, "per-term FP64 kernels not stored");
    if (term < 0 || term >= P->nterms) return fail(DCPSE_ERR_ARG, "term out of range");
    if (P->n > 0 && (!d_f || !d_out)) return fail(DCPSE_ERR_ARG, "NULL field");
    unsigned ord = 0;
    for (int d = 0; d < P->dim; ++d) ord += P->sigs[term][d];
    P->tstart(DCPSE_K_APPLY_TERM);
    cudaError_t e = apply_term_f64(P->n, P->rowptr, P->cols, P->k_term + (size_t)term * P->nnz,
                                   P->eip_group + (size_t)P->term_group[term] * P->n, ord, d_f, d_out, 0, P->stream);
    P->tstop(DCPSE_K_APPLY_TERM);
    DCPSE_CK(e);
    return DCPSE_OK;
}

int dcpse_apply_output_f64(dcpse_plan_t* P, int output, const double* d_f, double* d_out) {
    if (int rc = check_plan(P)) return rc;
    if (int rc = check_single_set(P)) return rc;
    if (!P->assembled || !P->k_term) return fail(DCPSE_ERR_STATE, "per-term FP64 kernels not stored");
    if (output < 0 || output >= P->nout) return fail(DCPSE_ERR_ARG, "output out of range");
    if (P->n > 0 && (!d_f || !d_out)) return fail(DCPSE_ERR_ARG, "NULL field");
    int first = 1;
    for (int t = 0; t < P->nterms; ++t) {
        if (P->term_output[t] != output) continue;
        unsigned ord = 0;
        for (int d = 0; d < P->dim; ++d) ord += P->sigs[t][d];
        P->tstart(DCPSE_K_APPLY_TERM);
        cudaError_t e = apply_term_f64(P->n, P->rowptr, P->cols, P->k_term + (size_t)t * P->nnz,
                                       P->eip_group + (size_t)P->term_group[t] * P->n, ord, d_f, d_out,
                                       first ? 0 : 1, P->stream);
        P->tstop(DCPSE_K_APPLY_TERM);
        DCPSE_CK(e);
        first = 0;
    }
    return DCPSE_OK;
}

namespace {
// The FP32 output weights on the sliced ELL layout, built from the CSR
// weights on first use after each assembly.
// The sliced layout of the current list (row order, slice offsets, columns),
// built on first use after each assembly.
int ensure_sell_layout(dcpse_plan_t* P) {
    if (P->sell_cols || P->n == 0 || P->sell_no_room) return DCPSE_OK;
    const int64_t ns = sell_slices(P->n);
    int32_t* slen = nullptr;
    int64_t* tmp = nullptr;
    cudaError_t e = cudaSuccess;
    // Renumbering: with the particles' cell order (one set, from the
    // neighbour build) the layout takes it when the list's own numbering
    // scatters the field reads at least twice as far (sum over the entries
    // of |q - p| against |inv[q] - inv[p]|), or when asked to
    P->sell_perm = nullptr;
    P->loc_sum[0] = P->loc_sum[1] = 0;
    if (P->cell_order && !P->two_set() && !P->surface() && P->reorder >= 0) {
        unsigned long long* sums = nullptr;
        e = dalloc(&P->sell_inv, (size_t)P->n);
        if (e == cudaSuccess) e = invert_perm(P->cell_order, P->n, P->sell_inv, P->stream);
        if (e == cudaSuccess) e = dalloc(&sums, 2);
        if (e == cudaSuccess) e = sell_locality(P->rowptr, P->cols, P->n, P->sell_inv, sums, P->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(P->loc_sum, sums, sizeof P->loc_sum, cudaMemcpyDeviceToHost, P->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(P->stream);
        dfree(sums);
        if (e == cudaSuccess && (P->reorder > 0 || 2 * P->loc_sum[1] < P->loc_sum[0]))
            P->sell_perm = P->cell_order;
        else
            dfree(P->sell_inv);
    }
    if (e == cudaSuccess) e = dalloc(&P->sell_row, (size_t)ns * 32);
    if (e == cudaSuccess) e = dalloc(&P->sell_off, (size_t)ns + 1);
    if (e == cudaSuccess) e = dalloc(&slen, (size_t)ns);
    if (e == cudaSuccess) e = dalloc(&tmp, (size_t)scan_tmp_elems(ns));
    if (e == cudaSuccess) e = sell_order(P->rowptr, P->n, P->sell_row, slen, P->sell_off, tmp, P->stream, P->sell_perm);
    int64_t total = 0;
    std::vector<int32_t> hlen((size_t)ns);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&total, P->sell_off + ns, sizeof total, cudaMemcpyDeviceToHost, P->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(hlen.data(), slen, sizeof(int32_t) * ns, cudaMemcpyDeviceToHost, P->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(P->stream);
    dfree(slen);
    dfree(tmp);
    if (e == cudaSuccess) {
        // the share of warp time a window's barrier would idle: per window
        // 8 x its longest slice against the sum of its slices
        int64_t busy = 0, held = 0;
        for (int64_t w = 0; w < ns / 8; ++w) {
            int32_t mx = 0;
            for (int k = 0; k < 8; ++k) {
                busy += hlen[(size_t)(w * 8 + k)];
                mx = std::max(mx, hlen[(size_t)(w * 8 + k)]);
            }
            held += 8 * (int64_t)mx;
        }
        P->sell_idle = busy > 0 ? (double)(held - busy) / (double)busy : 0.0;
    }
    if (e == cudaSuccess) e = dalloc(&P->sell_cols, (size_t)total + kPad);
    if (e == cudaSuccess)
        e = sell_fill(P->rowptr, P->cols, nullptr, nullptr, P->nnz, P->nout, P->n, P->two_set() ? 0 : 1,
                      P->sell_row, P->sell_off, total, P->sell_cols, nullptr, nullptr, P->stream, P->sell_perm,
                      P->sell_perm ? P->sell_inv : nullptr);
    if (e == cudaSuccess) e = cudaStreamSynchronize(P->stream);
    if (e == cudaErrorMemoryAllocation) {
        // the layout does not fit: the CSR kernels serve
        P->free_sell();
        cudaGetLastError();
        P->sell_no_room = true;
        return DCPSE_OK;
    }
    if (e != cudaSuccess) {
        P->free_sell();
        return fail(DCPSE_ERR_CUDA, std::string("sliced ELL layout: ") + cudaGetErrorString(e));
    }
    P->sell_total = total;
    // the warp-scheduled kernels' slice counter, allocated here rather than
    // at the first apply (which may run inside a stream capture); without it
    // the window kernel serves
    if (!P->slice_counter && dalloc(&P->slice_counter, 1) != cudaSuccess) {
        cudaGetLastError();
        P->slice_counter = nullptr;
    }
    return DCPSE_OK;
}

// One set of weights on the sliced layout: a failed allocation leaves it
// absent (the CSR kernels serve), other errors fail.
extern "C++" template <typename Alloc, typename Fill, typename Release>
int sell_stream(dcpse_plan_t* P, const char* what, Alloc alloc, Fill fill, Release release) {
    cudaError_t e = alloc();
    if (e == cudaSuccess) e = fill();
    if (e == cudaSuccess) e = cudaStreamSynchronize(P->stream);
    if (e == cudaSuccess) return DCPSE_OK;
    release();
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        return DCPSE_OK;
    }
    return fail(DCPSE_ERR_CUDA, std::string(what) + cudaGetErrorString(e));
}

// The FP32 output weights on the sliced layout, built at assembly.
int ensure_sell(dcpse_plan_t* P) {
    if (P->sell_w || !P->w32) return DCPSE_OK;
    if (int rc = ensure_sell_layout(P)) return rc;
    if (!P->sell_cols) return DCPSE_OK;
    return sell_stream(
        P, "sliced ELL weights: ", [&] { return dalloc(&P->sell_w, (size_t)P->nout * P->sell_total + kPad); },
        [&] {
            return sell_fill(P->rowptr, P->cols, P->w32, nullptr, P->nnz, P->nout, P->n, P->two_set() ? 0 : 1,
                             P->sell_row, P->sell_off, P->sell_total, nullptr, P->sell_w, nullptr, P->stream,
                             P->sell_perm);
        },
        [&] { dfree(P->sell_w); });
}

// The FP64 summed weights on the sliced layout, built on the first batched
// FP64 apply.
int ensure_sell64(dcpse_plan_t* P) {
    if (P->sell_w64 || !P->w64) return DCPSE_OK;
    if (int rc = ensure_sell_layout(P)) return rc;
    if (!P->sell_cols) return DCPSE_OK;
    return sell_stream(
        P, "sliced ELL FP64 weights: ",
        [&] { return dalloc(&P->sell_w64, (size_t)P->nout * P->sell_total + kPad); },
        [&] {
            return sell_fill64(P->rowptr, P->w64, P->nnz, P->nout, P->n, P->sell_row, P->sell_off, P->sell_total,
                               P->sell_w64, P->stream, P->sell_perm);
        },
        [&] { dfree(P->sell_w64); });
}

// The bf16 residual streams on the sliced layout, built on the first apply
// that asks for them (the FP32 weights' layout must exist).
int ensure_sell_resid(dcpse_plan_t* P) {
    if (P->sell_r || !P->sell_w || !P->r16) return DCPSE_OK;
    return sell_stream(
        P, "sliced ELL residuals: ",
        [&] { return cudaMalloc(&P->sell_r, ((size_t)P->nout * P->sell_total + kPad) * 2); },
        [&] {
            return sell_fill(P->rowptr, P->cols, nullptr, P->r16, P->nnz, P->nout, P->n, P->two_set() ? 0 : 1,
                             P->sell_row, P->sell_off, P->sell_total, nullptr, nullptr, P->sell_r, P->stream,
                             P->sell_perm);
        },
        [&] {
            if (P->sell_r) cudaFree(P->sell_r);
            P->sell_r = nullptr;
        });
}

// The FP32 residual streams on the sliced layout (the second float of each
// weight pair), built on the first apply that asks for them.
int ensure_sell_pair(dcpse_plan_t* P) {
    if (P->sell_r32 || !P->sell_w || !P->r32) return DCPSE_OK;
    return sell_stream(
        P, "sliced ELL weight pairs: ",
        [&] { return dalloc(&P->sell_r32, (size_t)P->nout * P->sell_total + kPad); },
        [&] {
            // the residuals take the weight streams' path of the fill
            return sell_fill(P->rowptr, P->cols, P->r32, nullptr, P->nnz, P->nout, P->n, P->two_set() ? 0 : 1,
                             P->sell_row, P->sell_off, P->sell_total, nullptr, P->sell_r32, nullptr, P->stream,
                             P->sell_perm);
        },
        [&] { dfree(P->sell_r32); });
}

// The evict-first hint of the sliced kernels' streams: on a renumbered layout
// unless the apply configuration says otherwise.
int stream_hint(const dcpse_plan_t* P) {
    if (P->apply_mode & DCPSE_APPLY_STREAM_HINT_ON) return 1;
    if (P->apply_mode & DCPSE_APPLY_STREAM_HINT_OFF) return 0;
    return P->sell_perm ? 1 : 0;
}

// The slice counter of the warp-scheduled sliced kernels, or null for the
// window-per-block kernel: outputs in host memory (their scattered stores
// are slow over NVLink-C2C), DCPSE_APPLY_SLICE_WINDOWS, or a layout whose
// windows hold slices of nearly equal length.  Measured (kernel ms, windows
// against warps): 128^3 lattice, 6 % idle at the barrier: FP32 0.591 /
// 0.614, bf16 residual streams 0.880 / 0.958, weight pairs 1.035 / 1.10;
// graded 2D cloud, 37 % idle: 0.161 / 0.146, 0.232 / 0.213, 0.261 / 0.260.
constexpr double kSliceIdleWarps = 0.15;
unsigned* slice_counter(dcpse_plan_t* P, bool host_out) {
    if (host_out || (P->apply_mode & DCPSE_APPLY_SLICE_WINDOWS)) return nullptr;
    if (P->sell_idle < kSliceIdleWarps && !(P->apply_mode & DCPSE_APPLY_SLICE_WARPS)) return nullptr;
    return P->slice_counter;  // (allocated with the layout)
}

// The FP32 batched apply of rows [r0, r1) (0, 0: all rows) from the plan's
// split field into d_out ([n_outputs][n]; in host memory with host_out).
int apply_f32_rows(dcpse_plan_t* P, int precision, double* d_out, int64_t r0, int64_t r1,
                   cudaStream_t on = nullptr, bool comp_all = false, bool csr_only = false,
                   bool host_out = false) {
    cudaStream_t st = on ? on : P->stream;
    ApplyF32 ap{};
    ap.n = P->n;
    ap.nout = P->nout;
    ap.rowptr = P->rowptr;
    ap.cols = P->cols;
    ap.w = P->w32;
    ap.resid = (precision == DCPSE_F32_RESID) ? P->r16 : nullptr;
    ap.ws = P->nnz;
    ap.nnz = P->nnz;
    ap.maxk = P->maxk;
    ap.f2 = P->f2;
    ap.out = d_out;
    ap.err = P->d_err;
    ap.mode = P->apply_mode & 15;
    ap.lanes = P->apply_lanes;
    ap.row0 = r0;
    ap.row1 = r1;
    // compensated sums for outputs with a term of order >= 2 (their
    // first-order contributions cancel), or for all outputs on request
    ap.comp = 0;
    for (int t = 0; t < P->nterms; ++t) {
        unsigned ord = 0;
        for (int d = 0; d < P->dim; ++d) ord += P->sigs[t][d];
        if (ord >= 2) ap.comp |= 1u << P->term_output[t];
    }
    // the residual correction only pays off with compensated sums
    if ((P->apply_mode & DCPSE_APPLY_COMPENSATE_ALL) || precision == DCPSE_F32_RESID ||
        precision == DCPSE_F32_PAIR || comp_all)
        ap.comp = 0xffffffffu;
    // sliced ELL layout: rows in whole windows of 256
    // (the automatic schedule: 15 % faster than the CSR kernels at 128^3)
    const int64_t rr0 = r0, rr1 = r1 ? r1 : P->n;
    const int mode = P->apply_mode & 15;
    const bool resid = precision == DCPSE_F32_RESID;
    const bool pair = precision == DCPSE_F32_PAIR;
    if (!csr_only && (mode == 0 || mode == 4) && rr0 % 256 == 0 && (rr1 % 256 == 0 || rr1 == P->n)) {
        if (int rc = ensure_sell(P)) return rc;
        if (resid)
            if (int rc = ensure_sell_resid(P)) return rc;
        if (pair)
            if (int rc = ensure_sell_pair(P)) return rc;
    }
    // (a renumbered layout serves whole-list applies only: the split field
    // is then at positions)
    if (!csr_only && (mode == 0 || mode == 4) && P->sell_w && (!resid || P->sell_r) && (!pair || P->sell_r32) &&
        rr0 % 256 == 0 &&
        (rr1 % 256 == 0 || rr1 == P->n) && (!P->sell_perm || (rr0 == 0 && rr1 == P->n))) {
        SellArgs sa{};
        sa.perm = P->sell_perm;
        sa.stream = stream_hint(P);
        sa.n = P->n;
        sa.nslices = sell_slices(P->n);
        sa.srow = P->sell_row;
        sa.off = P->sell_off;
        sa.cols = P->sell_cols;
        sa.w = P->sell_w;
        sa.r = resid ? static_cast<const __nv_bfloat16*>(P->sell_r) : nullptr;
        sa.r32 = pair ? P->sell_r32 : nullptr;
        sa.total = P->sell_total;
        sa.f2 = P->f2;
        sa.fx = pair ? reinterpret_cast<const long long*>(P->f2) : nullptr;
        sa.fx_meta = pair ? P->fx_meta : nullptr;
        sa.out = d_out;
        sa.oos = P->n;
        sa.ors = 1;
        sa.w0 = rr0 / 256;
        sa.w1 = (rr1 + 255) / 256;
        // a row's entries are summed by one thread: the compensated sum for
        // every output keeps first-order outputs at the CSR kernel's accuracy
        // (128^3 gradient: 5e-7 plain, ~1e-7 compensated; 1.5 % slower)
        sa.comp = 0xffffffffu;
        sa.no_self = 0;
        // (row chunks on their own streams run concurrently: one counter
        // per plan serves calls on the plan's stream only)
        sa.counter = on ? nullptr : slice_counter(P, host_out);
        P->tstart(DCPSE_K_APPLY_BATCHED, st);
        cudaError_t e = apply_sell(sa, P->nout, st);
        P->tstop(DCPSE_K_APPLY_BATCHED, st);
        DCPSE_CK(e);
        return DCPSE_OK;
    }
    // the weight pairs run on the sliced layout only (their field is in fixed point)
    if (pair) return fail(DCPSE_ERR_STATE, "DCPSE_F32_PAIR needs the sliced layout");
    P->tstart(DCPSE_K_APPLY_BATCHED, st);
    cudaError_t e = apply_batched_f32x(ap, st);
    P->tstop(DCPSE_K_APPLY_BATCHED, st);
    if (e == cudaErrorInvalidConfiguration && (P->apply_mode & 15) == 2)
        return fail(DCPSE_ERR_CAPACITY, "TMA-staged tiles of this plan do not fit in shared memory "
                                        "(fewer lanes per row or another mode)");
    DCPSE_CK(e);
    return DCPSE_OK;
}

int check_f32_weights(dcpse_plan_t* P, int precision) {
    if (!P->w32) return fail(DCPSE_ERR_STATE, "FP32 weights not stored");
    if (precision == DCPSE_F32_RESID && !P->r16)
        return fail(DCPSE_ERR_STATE, "FP32 residuals not stored (DCPSE_STORE_OUT_F32_RESID)");
    if ((precision == DCPSE_F32_BUDGET || precision == DCPSE_F32_PAIR) && !P->r32)
        return fail(DCPSE_ERR_STATE, "FP32 residuals not stored (DCPSE_STORE_OUT_F32_CORR)");
    if (precision == DCPSE_F32_BUDGET && P->budget_pass == DCPSE_F32_RESID && !P->r16)
        return fail(DCPSE_ERR_STATE, "the bf16 first pass needs DCPSE_STORE_OUT_F32_RESID");
    return DCPSE_OK;
}

// Whether a whole-list FP32 apply of this precision runs the sliced kernel
// (its layout and streams are built on first use).
int sell_ready(dcpse_plan_t* P, int precision, bool* ready) {
    *ready = false;
    const int mode = P->apply_mode & 15;
    if (mode != 0 && mode != 4) return DCPSE_OK;
    if (int rc = ensure_sell(P)) return rc;
    const bool resid = precision == DCPSE_F32_RESID || (precision == DCPSE_F32_BUDGET && P->budget_pass == DCPSE_F32_RESID);
    const bool pair = precision == DCPSE_F32_PAIR;
    if (resid)
        if (int rc = ensure_sell_resid(P)) return rc;
    if (pair)
        if (int rc = ensure_sell_pair(P)) return rc;
    *ready = P->sell_w && (!resid || P->sell_r) && (!pair || P->sell_r32);
    return DCPSE_OK;
}

// The split of a whole-list FP32 apply's field, at positions when the sliced
// kernel will run on a renumbered layout.
int split_for_apply(dcpse_plan_t* P, const double* d_f, int precision) {
    bool ready = false;
    if (int rc = sell_ready(P, precision, &ready)) return rc;
    return split_into_plan(P, d_f, P->n, 1, (ready && P->sell_perm) ? P->sell_inv : nullptr);
}

// The budget-driven FP32 apply of every row from the plan's split field into
// d_out ([n_outputs][n]): the sliced FP32 kernel with its weight-rounding
// bounds, then the FP64 residual correction of the rows whose bound exceeds
// the budget (every row when the sliced layout is not available).  With the
// DCPSE_F32_RESID first pass (dcpse_plan_set_error_budget) it adds the bf16
// residual streams: its bound is 2^8 times smaller, so far fewer rows need
// the second pass (worth it where many rows would, e.g. second derivatives
// on strongly graded clouds).
int apply_budget(dcpse_plan_t* P, double* d_out, bool host_out = false) {
    cudaStream_t st = P->stream;
    const int64_t n = P->n;
    if (n == 0) return DCPSE_OK;
    if (!P->maxabs) DCPSE_CK(dalloc(&P->maxabs, kMaxOutputs + 1));
    if (P->bnd_len < (int64_t)P->nout * n) {
        dfree(P->bnd);
        dfree(P->blist);
        P->bnd_len = 0;
        DCPSE_CK(dalloc(&P->bnd, (size_t)P->nout * n));
        DCPSE_CK(dalloc(&P->blist, (size_t)n));
        P->bnd_len = (int64_t)P->nout * n;
    }
    // the largest |output| per output and the list length start at zero
    DCPSE_CK(cudaMemsetAsync(P->maxabs, 0, sizeof(unsigned) * (kMaxOutputs + 1), st));
    if (!P->budget_count) {
        DCPSE_CK(dalloc(&P->budget_count, 1));
        DCPSE_CK(cudaMemsetAsync(P->budget_count, 0, sizeof(unsigned long long), st));
    }
    bool bounded = false, with_r16 = false, ready = false;
    if (int rc = sell_ready(P, DCPSE_F32_BUDGET, &ready)) return rc;
    {
        if (ready) {
            with_r16 = P->budget_pass == DCPSE_F32_RESID;
            SellArgs sa{};
            sa.perm = P->sell_perm;
            sa.stream = stream_hint(P);
            sa.n = n;
            sa.nslices = sell_slices(n);
            sa.srow = P->sell_row;
            sa.off = P->sell_off;
            sa.cols = P->sell_cols;
            sa.w = P->sell_w;
            sa.r = with_r16 ? static_cast<const __nv_bfloat16*>(P->sell_r) : nullptr;
            sa.total = P->sell_total;
            sa.f2 = P->f2;
            sa.out = d_out;
            sa.oos = n;
            sa.ors = 1;
            sa.w0 = 0;
            sa.w1 = (n + 255) / 256;
            sa.comp = 0xffffffffu;
            sa.no_self = 0;
            sa.bnd = P->bnd;
            sa.maxabs = P->maxabs;
            sa.counter = slice_counter(P, host_out);
            P->tstart(DCPSE_K_APPLY_BATCHED, st);
            cudaError_t e = apply_sell(sa, P->nout, st);
            P->tstop(DCPSE_K_APPLY_BATCHED, st);
            DCPSE_CK(e);
            bounded = true;
        }
    }
    if (!bounded)
        if (int rc = apply_f32_rows(P, DCPSE_F32, d_out, 0, 0, nullptr, true, true)) return rc;
    BudgetArgs b{};
    b.n = n;
    b.rowptr = P->rowptr;
    b.cols = P->cols;
    b.r32 = P->r32;
    b.r16 = with_r16 ? P->r16 : nullptr;
    b.ws = P->nnz;
    b.f2 = P->f2;
    b.out = d_out;
    b.oos = n;
    b.ors = 1;
    b.bnd = P->bnd;
    b.maxabs = P->maxabs;
    b.budget = P->budget;
    b.bound_scale = with_r16 ? 0x1p-32 : 0x1p-24;
    b.flag_all = bounded ? 0 : 1;
    b.count = P->budget_count;
    b.list = P->blist;
    b.list_len = P->maxabs + kMaxOutputs;
    b.inv = bounded ? (P->sell_perm ? P->sell_inv : nullptr) : nullptr;
    P->tstart(DCPSE_K_CORRECT, st);
    cudaError_t e = budget_correct(b, P->nout, st);
    P->tstop(DCPSE_K_CORRECT, st);
    DCPSE_CK(e);
    return DCPSE_OK;
}

}  // namespace

int dcpse_apply_batched(dcpse_plan_t* P, const double* d_f, double* d_out, int precision) {
    if (int rc = check_plan(P)) return rc;
    if (int rc = check_single_set(P)) return rc;
    if (!P->assembled) return fail(DCPSE_ERR_STATE, "not assembled");
    if (P->n > 0 && (!d_f || !d_out)) return fail(DCPSE_ERR_ARG, "NULL field");
    if (precision == DCPSE_F32_PAIR) {
        // FP64-class weights as float pairs on the sliced layout; without it
        // (no room, or a CSR schedule) the batched FP64 apply serves
        if (int rc = check_f32_weights(P, precision)) return rc;
        bool ready = false;
        if (int rc = sell_ready(P, precision, &ready)) return rc;
        if (ready) {
            if (int rc = fixed_into_plan(P, d_f, P->sell_perm ? P->sell_inv : nullptr)) return rc;
            return apply_f32_rows(P, precision, d_out, 0, 0);
        }
        precision = DCPSE_F64;
    }
    if (precision == DCPSE_F32 || precision == DCPSE_F32_RESID) {
        if (int rc = check_f32_weights(P, precision)) return rc;
        if (int rc = split_for_apply(P, d_f, precision)) return rc;
        return apply_f32_rows(P, precision, d_out, 0, 0);
    } else if (precision == DCPSE_F32_BUDGET) {
        if (int rc = check_f32_weights(P, precision)) return rc;
        if (int rc = split_for_apply(P, d_f, precision)) return rc;
        return apply_budget(P, d_out);
    } else if (precision == DCPSE_F64) {
        if (!P->w64) return fail(DCPSE_ERR_STATE, "FP64 output weights not stored");
        const int mode = P->apply_mode & 15;
        if (mode == 0 || mode == 4) {
            if (int rc = ensure_sell64(P)) return rc;
            if (P->sell_w64 && P->sell_perm && P->n > 0) {
                // a renumbered layout reads the field at positions
                if (P->fperm_len < P->n) {
                    dfree(P->fperm);
                    P->fperm_len = 0;
                    DCPSE_CK(dalloc(&P->fperm, (size_t)P->n));
                    P->fperm_len = P->n;
                }
                DCPSE_CK(permute_f64(d_f, P->n, P->sell_inv, P->fperm, P->stream));
            }
            if (P->sell_w64) {
                Sell64Args sa{};
                sa.perm = P->sell_perm;
                sa.stream = stream_hint(P);
                sa.n = P->n;
                sa.nwin = (P->n + 255) / 256;
                sa.srow = P->sell_row;
                sa.off = P->sell_off;
                sa.cols = P->sell_cols;
                sa.w = P->sell_w64;
                sa.total = P->sell_total;
                sa.f = P->sell_perm ? P->fperm : d_f;
                sa.fs = 1;
                sa.out = d_out;
                sa.oos = P->n;
                sa.ors = 1;
                P->tstart(DCPSE_K_APPLY_BATCHED);
                cudaError_t e = apply_sell64(sa, P->nout, P->stream);
                P->tstop(DCPSE_K_APPLY_BATCHED);
                DCPSE_CK(e);
                return DCPSE_OK;
            }
        }
        P->tstart(DCPSE_K_APPLY_BATCHED);
        cudaError_t e = apply_batched_f64(P->n, P->nout, P->rowptr, P->cols, P->w64, P->nnz, d_f, d_out, P->stream);
        P->tstop(DCPSE_K_APPLY_BATCHED);
        DCPSE_CK(e);
    } else {
        return fail(DCPSE_ERR_ARG,
                    "precision must be DCPSE_F32, DCPSE_F32_RESID, DCPSE_F32_BUDGET, DCPSE_F32_PAIR or DCPSE_F64");
    }
    return DCPSE_OK;
}

int dcpse_plan_set_error_budget(dcpse_plan_t* P, double rel, int first_pass) {
    if (int rc = check_plan(P)) return rc;
    if (!(rel > 0.0) || !(rel < 1.0)) return fail(DCPSE_ERR_ARG, "the error budget must lie in (0, 1)");
    if (first_pass != DCPSE_F32 && first_pass != DCPSE_F32_RESID)
        return fail(DCPSE_ERR_ARG, "the first pass must be DCPSE_F32 or DCPSE_F32_RESID");
    P->budget = rel;
    P->budget_pass = first_pass;
    return DCPSE_OK;
}

int dcpse_plan_assembly_info(dcpse_plan_t* P, int* gram_on_tensor_cores) {
    if (int rc = check_plan(P)) return rc;
    if (!gram_on_tensor_cores) return fail(DCPSE_ERR_ARG, "NULL output");
    *gram_on_tensor_cores = P->asm_tc ? 1 : 0;
    return DCPSE_OK;
}

int dcpse_plan_set_reorder(dcpse_plan_t* P, int policy) {
    if (int rc = check_plan(P)) return rc;
    if (policy < -1 || policy > 1) return fail(DCPSE_ERR_ARG, "policy must be -1, 0 or 1");
    if (policy != P->reorder) {
        P->reorder = policy;
        // the sliced layouts are rebuilt on next use
        const bool had = P->sell_w != nullptr;
        P->free_sell();
        if (had && P->assembled)
            if (int rc = ensure_sell(P)) return rc;
    }
    return DCPSE_OK;
}

int dcpse_plan_set_reorder_order(dcpse_plan_t* P, int order) {
    if (int rc = check_plan(P)) return rc;
    if (order < 0 || order > 1) return fail(DCPSE_ERR_ARG, "order must be 0 (Z-order of cells) or 1 (row-major)");
    P->reorder_order = order;  // used by the next neighbour build
    return DCPSE_OK;
}

int dcpse_plan_reorder_info(dcpse_plan_t* P, int* renumbered, double* mean_dist_list, double* mean_dist_cells) {
    if (int rc = check_plan(P)) return rc;
    if (renumbered) *renumbered = P->sell_perm ? 1 : 0;
    const double m = P->nnz > 0 ? (double)P->nnz : 1.0;
    if (mean_dist_list) *mean_dist_list = (double)P->loc_sum[0] / m;
    if (mean_dist_cells) *mean_dist_cells = (double)P->loc_sum[1] / m;
    return DCPSE_OK;
}

int dcpse_plan_budget_stats(dcpse_plan_t* P, int64_t* pairs_corrected, int reset) {
    if (int rc = check_plan(P)) return rc;
    if (!pairs_corrected) return fail(DCPSE_ERR_ARG, "NULL output");
    unsigned long long h = 0;
    if (P->budget_count) {
        DCPSE_CK(cudaMemcpyAsync(&h, P->budget_count, sizeof h, cudaMemcpyDeviceToHost, P->stream));
        DCPSE_CK(cudaStreamSynchronize(P->stream));
        if (reset) DCPSE_CK(cudaMemsetAsync(P->budget_count, 0, sizeof h, P->stream));
    }
    *pairs_corrected = (int64_t)h;
    return DCPSE_OK;
}

namespace {
// Device address of a pinned host buffer with a device mapping (cudaHostAlloc
// / cudaHostRegister), or null for pageable memory.
double* mapped_host(const void* h) {
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, h) == cudaSuccess && at.type == cudaMemoryTypeHost && at.devicePointer)
        return static_cast<double*>(at.devicePointer);
    cudaGetLastError();  // an unregistered pointer is not an error here
    return nullptr;
}

// streams and events of the pipelined host-buffer apply (created once)
int ensure_host_pipeline(dcpse_plan_t* P) {
    if (P->copy_stream) return DCPSE_OK;
    cudaError_t e = cudaStreamCreateWithFlags(&P->copy_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&P->h2d_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&P->apply2_stream, cudaStreamNonBlocking);
    for (int c = 0; c < kHostChunks && e == cudaSuccess; ++c) {
        e = cudaEventCreateWithFlags(&P->chunk_ev[c], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&P->piece_ev[c], cudaEventDisableTiming);
    }
    if (e != cudaSuccess) {
        for (int c = 0; c < kHostChunks; ++c) {
            if (P->chunk_ev[c]) cudaEventDestroy(P->chunk_ev[c]);
            if (P->piece_ev[c]) cudaEventDestroy(P->piece_ev[c]);
            P->chunk_ev[c] = P->piece_ev[c] = nullptr;
        }
        if (P->copy_stream) cudaStreamDestroy(P->copy_stream);
        if (P->h2d_stream) cudaStreamDestroy(P->h2d_stream);
        if (P->apply2_stream) cudaStreamDestroy(P->apply2_stream);
        P->copy_stream = P->h2d_stream = P->apply2_stream = nullptr;
        return fail(DCPSE_ERR_CUDA, cudaGetErrorString(e));
    }
    return DCPSE_OK;
}

// largest field index read by each row chunk, for the current list
int ensure_chunk_reach(dcpse_plan_t* P) {
    const ChunkBounds cb = make_chunk_bounds(P->n, f32_rows_per_wave(P->n, P->nnz, P->apply_lanes));
    bool same = P->reach_version == P->list_version && cb.nch == P->chunks.nch;
    for (int c = 0; same && c <= cb.nch; ++c) same = cb.b[c] == P->chunks.b[c];
    if (same) return DCPSE_OK;
    unsigned long long* d = nullptr;
    DCPSE_CK(dalloc(&d, kHostChunks));
    cudaError_t e = cudaMemsetAsync(d, 0, sizeof(unsigned long long) * kHostChunks, P->stream);
    if (e == cudaSuccess) {
        chunk_reach_kernel<<<std::max(1, std::min(num_sms() * 8, (int)((P->n + 255) / 256))), 256, 0, P->stream>>>(
            P->rowptr, P->cols, P->n, cb, d);
        e = cudaGetLastError();
    }
    unsigned long long h[kHostChunks] = {};
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, d, sizeof h, cudaMemcpyDeviceToHost, P->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(P->stream);
    dfree(d);
    DCPSE_CK(e);
    for (int c = 0; c < kHostChunks; ++c) P->chunk_reach[c] = (int64_t)h[c];
    P->chunks = cb;
    P->reach_version = P->list_version;
    return DCPSE_OK;
}
}  // namespace

int dcpse_apply_batched_host(dcpse_plan_t* P, const double* h_f, double* h_out, int precision) {
    if (int rc = check_plan(P)) return rc;
    if (int rc = check_single_set(P)) return rc;
    if (!P->assembled) return fail(DCPSE_ERR_STATE, "not assembled");
    if (P->n > 0 && (!h_f || !h_out)) return fail(DCPSE_ERR_ARG, "NULL field");
    // staging for pageable buffers, sized for the current particle count
    // (a new neighbour list may have more particles than the last call saw)
    if (P->hf_len < P->n || !P->hf) {
        dfree(P->hf);
        dfree(P->hout);
        P->hf_len = 0;
        DCPSE_CK(dalloc(&P->hf, P->n));
        DCPSE_CK(dalloc(&P->hout, (size_t)P->nout * P->n));
        P->hf_len = P->n;
    }
    const bool f32 = precision == DCPSE_F32 || precision == DCPSE_F32_RESID;
    if (precision == DCPSE_F32_BUDGET && P->n > 0) {
        // pinned field and outputs: the split reads the field in place, the
        // FP32 kernel and the correction write the outputs in place
        double* om = mapped_host(h_out);
        const double* fm = om ? mapped_host(h_f) : nullptr;
        if (om && fm) {
            if (int rc = check_f32_weights(P, precision)) return rc;
            if (int rc = split_for_apply(P, fm, precision)) return rc;
            if (int rc = apply_budget(P, om, true)) return rc;
            DCPSE_CK(cudaStreamSynchronize(P->stream));
            return DCPSE_OK;
        }
    }
    if (!f32 || (P->apply_mode & 15) == 2 || P->n < kHostChunkMinRows) {
        DCPSE_CK(cudaMemcpyAsync(P->hf, h_f, sizeof(double) * P->n, cudaMemcpyHostToDevice, P->stream));
        int rc = dcpse_apply_batched(P, P->hf, P->hout, precision);
        if (rc != DCPSE_OK) return rc;
        DCPSE_CK(cudaMemcpyAsync(h_out, P->hout, sizeof(double) * P->nout * P->n, cudaMemcpyDeviceToHost,
                                 P->stream));
        return dcpse_plan_check(P);
    }
    // Pipelined: the field goes up in kHostChunks pieces (copy + split on
    // h2d_stream, pieces and row chunks share the bounds); row chunk c
    // starts once the pieces up to its largest read
    // index have arrived; its outputs go back on copy_stream while later
    // chunks run.
    if (int rc = check_f32_weights(P, precision)) return rc;
    if (int rc = ensure_host_pipeline(P)) return rc;
    if (int rc = ensure_chunk_reach(P)) return rc;
    const int64_t n = P->n;
    if (P->f2_len < n) {
        dfree(P->f2);
        P->f2_len = 0;
        DCPSE_CK(dalloc(&P->f2, (size_t)n));
        P->f2_len = n;
    }
    // Pinned host outputs with a device mapping (cudaHostAlloc /
    // cudaHostRegister; over NVLink-C2C the GPU stores into them at full
    // rate): the apply writes them directly, with no copies back and only
    // three row chunks (for the upload of the field)
    auto mapped = [](const void* h) -> void* {
        cudaPointerAttributes at{};
        if (cudaPointerGetAttributes(&at, h) == cudaSuccess && at.type == cudaMemoryTypeHost && at.devicePointer)
            return at.devicePointer;
        cudaGetLastError();  // an unregistered pointer is not an error here
        return nullptr;
    };
    double* out_mapped = static_cast<double*>(mapped(h_out));
    const double* f_mapped = out_mapped ? static_cast<const double*>(mapped(h_f)) : nullptr;
    if (out_mapped && f_mapped) {
        // The field is pinned too: one split kernel reads it in place, then
        // one apply of all rows stores the outputs (128^3: 0.68 ms; splitting
        // the field in two pieces, the second beside the apply of the first
        // rows, took 0.71-0.74 ms for any first-row share from 1/32 to 1/4)
        if (int rc = split_for_apply(P, f_mapped, precision)) return rc;
        if (int rc = apply_f32_rows(P, precision, out_mapped, 0, 0, nullptr, false, false, true)) return rc;
        // the direct kernels report no device errors: a synchronisation of
        // the plan's stream puts the outputs in place
        DCPSE_CK(cudaStreamSynchronize(P->stream));
        return DCPSE_OK;
    }
    // earlier work of the plan's stream on these buffers comes first
    DCPSE_CK(cudaEventRecord(P->chunk_ev[0], P->stream));
    DCPSE_CK(cudaStreamWaitEvent(P->h2d_stream, P->chunk_ev[0], 0));
    DCPSE_CK(cudaStreamWaitEvent(P->apply2_stream, P->chunk_ev[0], 0));
    // pieces are issued just ahead of the first chunk that reads them, so the
    // first chunk's launch is not queued behind the whole upload
    const ChunkBounds& cb = P->chunks;
    const int nch = cb.nch;
    int issued = -1, waited[2] = {-1, -1};
    auto issue_piece = [&](int i) -> cudaError_t {
        const int64_t i0 = cb.b[i], i1 = cb.b[i + 1];
        cudaError_t e = cudaMemcpyAsync(P->hf + i0, h_f + i0, sizeof(double) * (size_t)(i1 - i0),
                                        cudaMemcpyHostToDevice, P->h2d_stream);
        if (e == cudaSuccess) e = split_f64(P->hf + i0, i1 - i0, P->f2 + i0, P->h2d_stream);
        if (e == cudaSuccess) e = cudaEventRecord(P->piece_ev[i], P->h2d_stream);
        return e;
    };
    if (out_mapped) {
        // row chunks = pieces [0, 1), [1, 3), [3, nch): the first starts after
        // a short upload, the last is one kernel for the bulk of the rows
        const int groups[4] = {0, std::min(1, nch), std::min(3, nch), nch};
        for (int gi = 0; gi < 3; ++gi) {
            const int c0 = groups[gi], c1 = groups[gi + 1];
            if (c0 >= c1) continue;
            int64_t reach = 0;
            for (int c = c0; c < c1; ++c) reach = std::max(reach, P->chunk_reach[c]);
            int need = 0;
            while (need + 1 < nch && cb.b[need + 1] <= reach) ++need;
            const int upto = std::min(nch - 1, std::max(need, c1));
            while (issued < upto) DCPSE_CK(issue_piece(++issued));
            if (need > waited[0]) {
                DCPSE_CK(cudaStreamWaitEvent(P->stream, P->piece_ev[need], 0));
                waited[0] = need;
            }
            if (int rc = apply_f32_rows(P, precision, out_mapped, cb.b[c0], cb.b[c1], nullptr, false, false, true)) {
                cudaStreamSynchronize(P->h2d_stream);
                return rc;
            }
        }
        while (issued < nch - 1) DCPSE_CK(issue_piece(++issued));
        DCPSE_CK(cudaStreamSynchronize(P->h2d_stream));
        DCPSE_CK(cudaStreamSynchronize(P->stream));
        return DCPSE_OK;
    }
    for (int c = 0; c < nch; ++c) {
        const int64_t r0 = cb.b[c], r1 = cb.b[c + 1];
        // the piece holding the largest index this chunk reads
        int need = 0;
        while (need + 1 < nch && cb.b[need + 1] <= P->chunk_reach[c]) ++need;
        // one piece of look-ahead keeps the copy engine busy
        const int upto = std::min(nch - 1, std::max(need, c + 1));
        while (issued < upto) DCPSE_CK(issue_piece(++issued));
        // consecutive chunks alternate between two streams (they are
        // independent), so one chunk's last blocks overlap the next one's
        // first instead of draining the GPU at every kernel boundary
        const int sid = c & 1;
        cudaStream_t cs = sid ? P->apply2_stream : P->stream;
        if (need > waited[sid]) {
            DCPSE_CK(cudaStreamWaitEvent(cs, P->piece_ev[need], 0));
            waited[sid] = need;
        }
        if (int rc = apply_f32_rows(P, precision, P->hout, r0, r1, cs)) {
            cudaStreamSynchronize(P->h2d_stream);
            cudaStreamSynchronize(P->apply2_stream);
            cudaStreamSynchronize(P->copy_stream);
            return rc;
        }
        DCPSE_CK(cudaEventRecord(P->chunk_ev[c], cs));
        DCPSE_CK(cudaStreamWaitEvent(P->copy_stream, P->chunk_ev[c], 0));
        // rows [r0, r1) of every output: one strided copy
        DCPSE_CK(cudaMemcpy2DAsync(h_out + r0, sizeof(double) * (size_t)n, P->hout + r0, sizeof(double) * (size_t)n,
                                   sizeof(double) * (size_t)(r1 - r0), (size_t)P->nout, cudaMemcpyDeviceToHost,
                                   P->copy_stream));
    }
    while (issued < nch - 1) DCPSE_CK(issue_piece(++issued));
    // rows never wait on pieces beyond their reach; the last piece must
    // still be done before the call returns (the copy stream waited for
    // every chunk, on both apply streams)
    DCPSE_CK(cudaStreamSynchronize(P->h2d_stream));
    DCPSE_CK(cudaStreamSynchronize(P->copy_stream));
    return dcpse_plan_check(P);
}

int dcpse_p2p_f64(dcpse_plan_t* P, int term, const double* d_f_support, int ncomp, double* d_out) {
    if (int rc = check_plan(P)) return rc;
    if (!P->assembled || !P->k_term) return fail(DCPSE_ERR_STATE, "per-term FP64 kernels not stored");
    if (term < 0 || term >= P->nterms) return fail(DCPSE_ERR_ARG, "term out of range");
    if (ncomp < 1) return fail(DCPSE_ERR_ARG, "ncomp must be >= 1");
    if ((P->two_set() ? P->n_sup : P->n) > 0 && !d_f_support) return fail(DCPSE_ERR_ARG, "NULL field");
    if (P->n > 0 && !d_out) return fail(DCPSE_ERR_ARG, "NULL output");
    P->tstart(DCPSE_K_APPLY_TERM);
    cudaError_t e = p2p_f64(P->n, P->rowptr, P->cols, P->k_term + (size_t)term * P->nnz,
                            P->eip_group + (size_t)P->term_group[term] * P->n, ncomp, d_f_support, d_out, P->stream);
    P->tstop(DCPSE_K_APPLY_TERM);
    DCPSE_CK(e);
    return DCPSE_OK;
}

int dcpse_p2p(dcpse_plan_t* P, const double* d_f_support, int ncomp, double* d_out, int precision) {
    if (int rc = check_plan(P)) return rc;
    if (!P->assembled) return fail(DCPSE_ERR_STATE, "not assembled");
    if (ncomp < 1) return fail(DCPSE_ERR_ARG, "ncomp must be >= 1");
    const int64_t nf = P->two_set() ? P->n_sup : P->n;
    if (nf > 0 && !d_f_support) return fail(DCPSE_ERR_ARG, "NULL field");
    if (P->n > 0 && !d_out) return fail(DCPSE_ERR_ARG, "NULL output");
    for (int c = 0; c < ncomp; ++c) {
        if (precision == DCPSE_F32) {
            if (!P->w32) return fail(DCPSE_ERR_STATE, "FP32 weights not stored");
            if (nf > 0)
                if (int rc = split_into_plan(P, d_f_support + c, nf, ncomp)) return rc;
            ApplyF32 ap{};
            ap.n = P->n;
            ap.nout = P->nout;
            ap.rowptr = P->rowptr;
            ap.cols = P->cols;
            ap.w = P->w32;
            ap.ws = P->nnz;
            ap.nnz = P->nnz;
            ap.maxk = P->maxk;
            ap.f2 = P->f2;
            ap.out = d_out + c;
            ap.oos = P->n * ncomp;
            ap.ors = ncomp;
            ap.err = P->d_err;
            ap.mode = P->apply_mode & 15;
            ap.lanes = P->apply_lanes;
            ap.comp = (P->apply_mode & DCPSE_APPLY_COMPENSATE_ALL) ? 0xffffffffu : 0u;
            ap.no_self = 1;
            const int mode = P->apply_mode & 15;
            if ((mode == 0 || mode == 4) && nf > 0) {
                if (int rc = ensure_sell(P)) return rc;
                if (P->sell_w && !P->sell_perm) {  // fields in list order
                    SellArgs sa{};
                    sa.n = P->n;
                    sa.nslices = sell_slices(P->n);
                    sa.srow = P->sell_row;
                    sa.off = P->sell_off;
                    sa.cols = P->sell_cols;
                    sa.w = P->sell_w;
                    sa.total = P->sell_total;
                    sa.f2 = P->f2;
                    sa.out = d_out + c;
                    sa.oos = P->n * ncomp;
                    sa.ors = ncomp;
                    sa.w0 = 0;
                    sa.w1 = (P->n + 255) / 256;
                    sa.comp = 0xffffffffu;  // one thread sums the whole row
                    sa.no_self = 1;
                    sa.counter = slice_counter(P, false);
                    P->tstart(DCPSE_K_APPLY_BATCHED);
                    cudaError_t e = apply_sell(sa, P->nout, P->stream);
                    P->tstop(DCPSE_K_APPLY_BATCHED);
                    DCPSE_CK(e);
                    continue;
                }
            }
            P->tstart(DCPSE_K_APPLY_BATCHED);
            cudaError_t e = apply_batched_f32x(ap, P->stream);
            P->tstop(DCPSE_K_APPLY_BATCHED);
            if (e == cudaErrorInvalidConfiguration && (P->apply_mode & 15) == 2)
                return fail(DCPSE_ERR_CAPACITY, "TMA-staged tiles of this plan do not fit in shared memory");
            DCPSE_CK(e);
        } else if (precision == DCPSE_F64) {
            if (!P->w64) return fail(DCPSE_ERR_STATE, "FP64 output weights not stored");
            const int mode = P->apply_mode & 15;
            if ((mode == 0 || mode == 4) && nf > 0) {
                if (int rc = ensure_sell64(P)) return rc;
                if (P->sell_w64 && !P->sell_perm) {  // fields in list order
                    Sell64Args sa{};
                    sa.n = P->n;
                    sa.nwin = (P->n + 255) / 256;
                    sa.srow = P->sell_row;
                    sa.off = P->sell_off;
                    sa.cols = P->sell_cols;
                    sa.w = P->sell_w64;
                    sa.total = P->sell_total;
                    sa.f = d_f_support + c;
                    sa.fs = ncomp;
                    sa.out = d_out + c;
                    sa.oos = P->n * ncomp;
                    sa.ors = ncomp;
                    sa.no_self = 1;
                    P->tstart(DCPSE_K_APPLY_BATCHED);
                    cudaError_t e = apply_sell64(sa, P->nout, P->stream);
                    P->tstop(DCPSE_K_APPLY_BATCHED);
                    DCPSE_CK(e);
                    continue;
                }
            }
            P->tstart(DCPSE_K_APPLY_BATCHED);
            cudaError_t e = apply_batched_f64(P->n, P->nout, P->rowptr, P->cols, P->w64, P->nnz,
                                              nf > 0 ? d_f_support + c : nullptr, d_out + c, P->stream, 1,
                                              P->n * ncomp, ncomp, ncomp);
            P->tstop(DCPSE_K_APPLY_BATCHED);
            DCPSE_CK(e);
        } else {
            return fail(DCPSE_ERR_ARG, "precision must be DCPSE_F32 or DCPSE_F64");
        }
    }
    return DCPSE_OK;
}

int dcpse_operator_csr(dcpse_plan_t* P, int output, double coeff, const int64_t* d_rows, int64_t n_rows, int nvar,
                       int var, int64_t* d_rowptr_out, int64_t* d_cols_out, double* d_vals_out, int64_t* nnz_out) {
    if (int rc = check_plan(P)) return rc;
    if (int rc = check_single_set(P)) return rc;
    if (!P->assembled || !P->k_term) return fail(DCPSE_ERR_STATE, "per-term FP64 kernels not stored");
    if (output < 0 || output >= P->nout) return fail(DCPSE_ERR_ARG, "output out of range");
    if (nvar < 1 || var < 0 || var >= nvar) return fail(DCPSE_ERR_ARG, "need 0 <= var < nvar");
    if (!nnz_out || !d_rowptr_out) return fail(DCPSE_ERR_ARG, "NULL row offsets or count");
    if (!d_rows) n_rows = P->n;
    if (n_rows < 0) return fail(DCPSE_ERR_ARG, "bad row count");
    if ((d_cols_out == nullptr) != (d_vals_out == nullptr)) return fail(DCPSE_ERR_ARG, "pass both or neither of cols/vals");
    cudaStream_t s = P->stream;
    if (d_rows && n_rows > 0) {
        unsigned long long* bad = nullptr;
        DCPSE_CK(dalloc(&bad, 1));
        cudaError_t e = cudaMemsetAsync(bad, 0, sizeof(unsigned long long), s);
        if (e == cudaSuccess) {
            index_check_kernel<<<std::max(1, (int)std::min<int64_t>(num_sms() * 8, (n_rows + 255) / 256)), 256, 0, s>>>(
                d_rows, n_rows, P->n, bad);
            e = cudaGetLastError();
        }
        unsigned long long hb = 0;
        if (e == cudaSuccess) e = cudaMemcpyAsync(&hb, bad, sizeof hb, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        dfree(bad);
        DCPSE_CK(e);
        if (hb) return fail(DCPSE_ERR_ARG, "row particle index out of range");
    }
    int32_t* counts = nullptr;
    int64_t* tmp = nullptr;
    cudaError_t e = dalloc(&counts, (size_t)std::max<int64_t>(n_rows, 1));
    if (e == cudaSuccess) e = dalloc(&tmp, (size_t)scan_tmp_elems(std::max<int64_t>(n_rows, 1)));
    if (e == cudaSuccess) e = csr_row_counts(P->rowptr, P->cols, d_rows, n_rows, counts, s);
    if (e == cudaSuccess) e = exclusive_scan_i32(counts, n_rows, d_rowptr_out, tmp, s);
    int64_t nnz = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&nnz, d_rowptr_out + n_rows, sizeof(int64_t), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    dfree(counts);
    dfree(tmp);
    DCPSE_CK(e);
    *nnz_out = nnz;
    if (!d_cols_out) return DCPSE_OK;
    MatArgs a{};
    a.rowptr = P->rowptr;
    a.cols = P->cols;
    a.rows = d_rows;
    a.nrows = n_rows;
    a.coeff = coeff;
    a.nvar = nvar;
    a.var = var;
    a.out_rowptr = d_rowptr_out;
    a.out_cols = d_cols_out;
    a.out_vals = d_vals_out;
    for (int t = 0; t < P->nterms; ++t) {
        if (P->term_output[t] != output) continue;
        unsigned ord = 0;
        for (int d = 0; d < P->dim; ++d) ord += P->sigs[t][d];
        a.K[a.nterms] = P->k_term + (size_t)t * P->nnz;
        a.eip[a.nterms] = P->eip_group + (size_t)P->term_group[t] * P->n;
        a.sign[a.nterms] = (ord % 2 == 0 && ord != 0) ? -1.0 : 1.0;
        a.nterms++;
    }
    DCPSE_CK(csr_fill(a, s));
    return DCPSE_OK;
}

int dcpse_plan_check(dcpse_plan_t* P) {
    if (int rc = check_plan(P)) return rc;
    int herr = 0;
    DCPSE_CK(cudaMemcpyAsync(&herr, P->d_err, sizeof(int), cudaMemcpyDeviceToHost, P->stream));
    DCPSE_CK(cudaStreamSynchronize(P->stream));
    if (herr) return fail(DCPSE_ERR_TIMEOUT, "a bounded device wait ran out; results of this plan are invalid");
    return DCPSE_OK;
}

int dcpse_plan_set_apply_config(dcpse_plan_t* P, int lanes, int mode) {
    if (int rc = check_plan(P)) return rc;
    if (lanes != 0 && lanes != 4 && lanes != 8 && lanes != 16 && lanes != 32)
        return fail(DCPSE_ERR_ARG, "lanes must be 0, 4, 8, 16 or 32");
    if ((mode & ~(15 | DCPSE_APPLY_COMPENSATE_ALL | DCPSE_APPLY_STREAM_HINT_ON | DCPSE_APPLY_STREAM_HINT_OFF |
                  DCPSE_APPLY_SLICE_WINDOWS | DCPSE_APPLY_SLICE_WARPS)) != 0 ||
        (mode & 15) > 4 || ((mode & DCPSE_APPLY_STREAM_HINT_ON) && (mode & DCPSE_APPLY_STREAM_HINT_OFF)) ||
        ((mode & DCPSE_APPLY_SLICE_WINDOWS) && (mode & DCPSE_APPLY_SLICE_WARPS)))
        return fail(DCPSE_ERR_ARG, "mode must be 0..4, optionally | DCPSE_APPLY_COMPENSATE_ALL, one "
                                   "DCPSE_APPLY_STREAM_HINT_* bit and one DCPSE_APPLY_SLICE_* bit");
    P->apply_lanes = lanes;
    P->apply_mode = mode;
    return DCPSE_OK;
}

int dcpse_plan_set_assembly_config(dcpse_plan_t* P, int bin_width, int warps, int qr_lanes) {
    if (int rc = check_plan(P)) return rc;
    if (bin_width < 0) return fail(DCPSE_ERR_ARG, "bin_width must be >= 0");
    if (warps != 2 && warps != 4 && warps != 8) return fail(DCPSE_ERR_ARG, "warps must be 2, 4 or 8");
    if (qr_lanes != 0 && qr_lanes != 1 && qr_lanes != 2 && qr_lanes != 4 && qr_lanes != 8 && qr_lanes != 16 &&
        qr_lanes != 32)
        return fail(DCPSE_ERR_ARG, "qr_lanes must be 0, 1, 2, 4, 8, 16 or 32");
    P->asm_bin_width = bin_width;
    P->asm_warps = warps;
    P->asm_qr_lanes = qr_lanes;
    return DCPSE_OK;
}

int dcpse_plan_set_timing(dcpse_plan_t* P, int enable) {
    if (int rc = check_plan(P)) return rc;
    P->timing = enable != 0;
    return DCPSE_OK;
}

int dcpse_plan_timing(dcpse_plan_t* P, int kernel, double* total_ms, int64_t* launches) {
    if (int rc = check_plan(P)) return rc;
    if (kernel < 0 || kernel >= DCPSE_K_COUNT) return fail(DCPSE_ERR_ARG, "kernel id out of range");
    DCPSE_CK(cudaStreamSynchronize(P->stream));
    double tot = 0.0;
    KernelTimer& T = P->timers[kernel];
    for (size_t i = 0; i < T.used; ++i) {
        float ms = 0.f;
        DCPSE_CK(cudaEventElapsedTime(&ms, T.ev[i].first, T.ev[i].second));
        tot += ms;
    }
    if (total_ms) *total_ms = tot;
    if (launches) *launches = (int64_t)T.used;
    return DCPSE_OK;
}

int dcpse_plan_reset_timing(dcpse_plan_t* P) {
    if (int rc = check_plan(P)) return rc;
    DCPSE_CK(cudaStreamSynchronize(P->stream));
    for (auto& T : P->timers) T.used = 0;
    return DCPSE_OK;
}

}  // extern "C"
