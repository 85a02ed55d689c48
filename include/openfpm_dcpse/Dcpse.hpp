// Dcpse.hpp -- drop-in for openfpm_numerics' Dcpse<dim, VerletList_type,
// vector_type> (src/DCPSE/Dcpse.hpp:43-826) on the GB300 C-ABI.
//
// Same constructor arguments, the same bulk and per-key
// computeDifferentialOperator, the same accessors (getNumNN, getCoeffNN,
// getIndexNN, getSign, getEpsilonInvPrefactor), initializeUpdate, save/load,
// checkMomenta and DrawKernel.  Assembly and application run on the GPU
// through include/openfpm_dcpse/dcpse_capi.h; the FP64 results are those of
// the reference algorithm in its operation order.  Host code here needs no
// CUDA headers: device memory goes through dcpse_device_alloc / dcpse_copy.
//
// The particle and Verlet-list types are template parameters, as in the
// reference; only these members are used:
//   particles.size_local(), particles.getPos(p)[d], particles.getProp<i>(p)
//   verletList.getNNPart(p), verletList.get(p, j)
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <functional>
#include <iostream>
#include <limits>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "dcpse_capi.h"
#include "particles.hpp"

namespace openfpm_dcpse {

// src/DCPSE/SupportBuilder.hpp:13-19
enum support_options { RADIUS, LOAD, ADAPTIVE, AT_LEAST_N_PARTICLES };

namespace detail {

inline void check(int rc, bool allow_particles = false) {
    if (rc == DCPSE_OK || (allow_particles && rc == DCPSE_ERR_PARTICLES)) return;
    throw std::runtime_error(std::string("DC-PSE: ") + dcpse_last_error());
}

// the C-ABI reads and writes as many values per field as the plan has
// particles: a property of another particle count (particles added or
// removed without update()) is refused
inline void check_rows(std::size_t rows, int64_t n) {
    if (n >= 0 && (int64_t)rows != n)
        throw std::invalid_argument("DC-PSE operator: the property has " + std::to_string(rows) +
                                    " values, the operator was built for " + std::to_string(n) +
                                    " particles (call update() after changing the particle set)");
}

// Device buffer owned by host code.
class DevBuf {
public:
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void* get() const { return p_; }
    void ensure(std::size_t bytes) {
        if (bytes <= bytes_) return;
        release();
        check(dcpse_device_alloc(&p_, bytes));
        bytes_ = bytes;
    }
    void upload(const void* h, std::size_t bytes) {
        ensure(bytes);
        check(dcpse_copy(p_, h, bytes));
    }
    void download(void* h, std::size_t bytes) const { check(dcpse_copy(h, p_, bytes)); }
    void release() {
        if (p_) dcpse_device_free(p_);
        p_ = nullptr;
        bytes_ = 0;
    }

private:
    void* p_ = nullptr;
    std::size_t bytes_ = 0;
};

// Page-locked (pinned) host buffer owned by host code: the batched applies
// read their field from it and write their outputs into it in place.
class PinBuf {
public:
    PinBuf() = default;
    PinBuf(const PinBuf&) = delete;
    PinBuf& operator=(const PinBuf&) = delete;
    ~PinBuf() { release(); }
    double* get() const { return static_cast<double*>(p_); }
    void ensure(std::size_t count) {
        if (count <= count_) return;
        release();
        check(dcpse_host_alloc(&p_, count * sizeof(double)));
        count_ = count;
    }
    void release() {
        if (p_) dcpse_host_free(p_);
        p_ = nullptr;
        count_ = 0;
    }

private:
    void* p_ = nullptr;
    std::size_t count_ = 0;
};

// Surface operator set-up (SurfaceDcpse, Dcpse.hpp:829-1085): unit normals
// of the support particles, nCount virtual particles per side at spacing
// nSpacing, and the cutoff / self option of the Verlet list handed in.
struct SurfaceCfg {
    bool on = false;
    std::vector<double> normals;
    std::function<std::vector<double>()> read_normals;  // normals of the current positions (updates)
    int n_count = 0;
    double spacing = 0.0;
    double rcut = 0.0;
    bool skip_ref = true;
    // support_options::ADAPTIVE: spacing along the normal per support particle
    // (property 0 / nCount) and the adaptive list's per-particle cutoffs
    std::vector<double> spacings;
    std::function<std::vector<double>()> read_spacings;
    std::vector<double> rcuts;
    std::function<std::vector<double>()> read_rcuts;

    // re-read what depends on the particles (an update after they moved)
    void refresh() {
        if (read_normals) normals = read_normals();
        if (read_spacings) spacings = read_spacings();
        if (read_rcuts) rcuts = read_rcuts();
    }
};

template <typename VL>
double list_rcut(const VL& vl, double fallback) {
    if constexpr (std::is_same<VL, VerletList>::value)
        return vl.rCut > 0.0 ? vl.rCut : fallback;
    else
        return fallback;
}

template <typename VL>
bool list_skip_ref(const VL& vl) {
    if constexpr (std::is_same<VL, VerletList>::value)
        return vl.skip_ref;
    else
        return true;
}

template <typename VL>
std::vector<double> list_rcuts(const VL& vl) {
    if constexpr (std::is_same<VL, VerletList>::value)
        return vl.rcuts;
    else
        return {};
}

template <unsigned int NORMAL_ID, typename Parts, typename VL>
SurfaceCfg surface_cfg(Parts& sup, const VL& vl, double rCut, double nSpacing, unsigned nCount,
                       support_options opt = support_options::RADIUS) {
    SurfaceCfg c;
    c.on = true;
    Parts* ps = &sup;
    if (opt == support_options::ADAPTIVE) {
        // nSpacing_p = property 0 / nCount (Dcpse.hpp:1055-1066); the support
        // of particle p reaches the cutoff of the adaptive list
        if (nCount == 0) throw std::invalid_argument("support_options::ADAPTIVE needs nCount > 0");
        c.read_spacings = [ps, nCount]() {
            std::vector<double> sp(ps->size_local());
            for (std::size_t p = 0; p < ps->size_local(); ++p)
                sp[p] = (double)ps->template getProp<0>(p) / (double)nCount;
            return sp;
        };
        c.spacings = c.read_spacings();
        const VL* pvl = &vl;
        c.read_rcuts = [pvl]() { return list_rcuts(*pvl); };
        c.rcuts = c.read_rcuts();
        if (c.rcuts.size() != sup.size_local())
            throw std::invalid_argument("support_options::ADAPTIVE needs an adaptive Verlet list (getVerletAdaptRCut)");
    }
    c.read_normals = [ps]() {
        const int dim = Parts::dims;
        std::vector<double> nrm(ps->size_local() * dim);
        for (std::size_t p = 0; p < ps->size_local(); ++p)
            for (int d = 0; d < dim; ++d) nrm[p * dim + d] = (double)ps->template getProp<NORMAL_ID>(p)[d];
        return nrm;
    };
    c.normals = c.read_normals();
    c.n_count = (int)nCount;
    c.spacing = nSpacing;
    c.rcut = list_rcut(vl, rCut);
    c.skip_ref = list_skip_ref(vl);
    return c;
}

// A plan plus the host <-> device staging of positions, lists and fields.
class PlanHost {
public:
    // outputs[o] = list of signatures (dim entries each) summed into output o
    PlanHost(int dim, const std::vector<std::vector<std::vector<unsigned>>>& outputs, unsigned order,
             double h_over_eps)
        : dim_(dim) {
        std::vector<int> terms;
        std::vector<unsigned> sigs;
        for (const auto& o : outputs) {
            terms.push_back((int)o.size());
            for (const auto& s : o) {
                unsigned ord = 0;
                for (int d = 0; d < dim; ++d) {
                    sigs.push_back(s[d]);
                    ord += s[d];
                }
                term_order_.push_back(ord);
            }
        }
        check(dcpse_plan_create(&plan_, dim, (int)outputs.size(), terms.data(), sigs.data(), order, h_over_eps));
        nout_ = (int)outputs.size();
    }
    PlanHost(const PlanHost&) = delete;
    PlanHost& operator=(const PlanHost&) = delete;
    ~PlanHost() {
        if (plan_) dcpse_plan_destroy(plan_);
    }

    dcpse_plan_t* plan() const { return plan_; }
    int64_t n() const { return n_; }
    int64_t nnz() const { return (int64_t)cols_.size(); }
    const std::vector<int64_t>& rowptr() const { return rowptr_; }
    const std::vector<int32_t>& cols() const { return cols_; }
    unsigned term_order(int t) const { return term_order_[t]; }
    int n_terms() const { return (int)term_order_.size(); }

    template <typename Parts, typename VL>
    void set_particles(Parts& parts, VL& vl) {
        set_particles(parts, parts, vl, false);
    }

    // two sets: rows are the domain particles, columns the support particles
    template <typename Sup, typename Dom, typename VL>
    void set_particles(Sup& sup, Dom& dom, VL& vl, bool two_set) {
        n_ = (int64_t)dom.size_local();
        n_sup_ = two_set ? (int64_t)sup.size_local() : n_;
        std::vector<double> pos((std::size_t)n_ * dim_);
        for (int64_t p = 0; p < n_; ++p)
            for (int d = 0; d < dim_; ++d) pos[(std::size_t)p * dim_ + d] = (double)dom.getPos(p)[d];
        pos_.upload(pos.data(), std::max<std::size_t>(pos.size(), 1) * sizeof(double));
        if (two_set) {
            std::vector<double> sp((std::size_t)n_sup_ * dim_);
            for (int64_t q = 0; q < n_sup_; ++q)
                for (int d = 0; d < dim_; ++d) sp[(std::size_t)q * dim_ + d] = (double)sup.getPos(q)[d];
            spos_.upload(sp.data(), std::max<std::size_t>(sp.size(), 1) * sizeof(double));
            check(dcpse_plan_set_support(plan_, (const double*)spos_.get(), n_sup_, 1));
        } else {
            check(dcpse_plan_set_support(plan_, nullptr, 0, 1));
        }
        rowptr_.assign((std::size_t)n_ + 1, 0);
        cols_.clear();
        for (int64_t p = 0; p < n_; ++p) {
            std::size_t k = vl.getNNPart((std::size_t)p);
            for (std::size_t j = 0; j < k; ++j) cols_.push_back((int32_t)vl.get((std::size_t)p, j));
            rowptr_[(std::size_t)p + 1] = (int64_t)cols_.size();
        }
        DevBuf drp, dcl;
        drp.upload(rowptr_.data(), rowptr_.size() * sizeof(int64_t));
        dcl.upload(cols_.data(), std::max<std::size_t>(cols_.size(), 1) * sizeof(int32_t));
        check(dcpse_set_neighbors(plan_, n_, (int64_t)cols_.size(), (const int64_t*)drp.get(),
                                  (const int32_t*)dcl.get()));
        cache_valid_ = false;
    }

    // returns the number of particles that could not be assembled
    int64_t assemble(int flags) {
        int rc = dcpse_assemble(plan_, (const double*)pos_.get(), nullptr, flags);
        check(rc, true);
        cache_valid_ = false;
        if (surface_) refresh_list();
        if (rc == DCPSE_ERR_PARTICLES) {
            int64_t nb = 0, first = -1;
            int code = 0;
            check(dcpse_particle_status(plan_, &nb, &first, &code));
            last_fail_code_ = code;
            return nb;
        }
        last_fail_code_ = 0;
        return 0;
    }
    int last_fail_code() const { return last_fail_code_; }

    // every output of the field f in one batched pass (precision DCPSE_F32,
    // DCPSE_F32_RESID or DCPSE_F32_BUDGET): f and the outputs go through
    // pinned staging buffers, which the kernels read and write in place;
    // out[o] gets output o
    void apply_batched(int precision, const double* f, std::vector<std::vector<double>>& out) {
        const std::size_t n = (std::size_t)std::max<int64_t>(n_, 0);
        pin_f_.ensure(std::max<std::size_t>(n, 1));
        pin_o_.ensure(std::max<std::size_t>(n * nout_, 1));
        std::copy(f, f + n, pin_f_.get());
        check(dcpse_apply_batched_host(plan_, pin_f_.get(), pin_o_.get(), precision));
        out.resize(nout_);
        for (int o = 0; o < nout_; ++o) out[o].assign(pin_o_.get() + o * n, pin_o_.get() + (o + 1) * n);
    }

    // FP64 output o of the field f (host arrays of n values)
    void apply_output(int o, const double* f, double* out) {
        fd_.upload(f, (std::size_t)n_ * sizeof(double));
        od_.ensure((std::size_t)std::max<int64_t>(n_, 1) * sizeof(double));
        check(dcpse_apply_output_f64(plan_, o, (const double*)fd_.get(), (double*)od_.get()));
        od_.download(out, (std::size_t)n_ * sizeof(double));
    }
    // surface operator: the device builds the lists over the support
    // extended along the normals and accumulates them at assembly
    template <typename Sup, typename Dom>
    void set_surface_particles(Sup& sup, Dom& dom, bool two_set, const SurfaceCfg& c) {
        n_ = (int64_t)dom.size_local();
        n_sup_ = two_set ? (int64_t)sup.size_local() : n_;
        std::vector<double> pos((std::size_t)n_ * dim_);
        for (int64_t p = 0; p < n_; ++p)
            for (int d = 0; d < dim_; ++d) pos[(std::size_t)p * dim_ + d] = (double)dom.getPos(p)[d];
        pos_.upload(pos.data(), std::max<std::size_t>(pos.size(), 1) * sizeof(double));
        if (two_set) {
            std::vector<double> sp((std::size_t)n_sup_ * dim_);
            for (int64_t q = 0; q < n_sup_; ++q)
                for (int d = 0; d < dim_; ++d) sp[(std::size_t)q * dim_ + d] = (double)sup.getPos(q)[d];
            spos_.upload(sp.data(), std::max<std::size_t>(sp.size(), 1) * sizeof(double));
        }
        nrm_.upload(c.normals.data(), std::max<std::size_t>(c.normals.size(), 1) * sizeof(double));
        check(dcpse_plan_set_support(plan_, two_set ? (const double*)spos_.get() : nullptr, two_set ? n_sup_ : 0,
                                     c.skip_ref ? 1 : 0));
        const double* d_spacings = nullptr;
        if (!c.spacings.empty()) {
            spc_.upload(c.spacings.data(), c.spacings.size() * sizeof(double));
            d_spacings = (const double*)spc_.get();
        }
        check(dcpse_plan_set_surface(plan_, (const double*)nrm_.get(), c.n_count, c.spacing, d_spacings));
        const double* d_rcuts = nullptr;
        if (!c.rcuts.empty()) {
            rcs_.upload(c.rcuts.data(), c.rcuts.size() * sizeof(double));
            d_rcuts = (const double*)rcs_.get();
        }
        check(dcpse_build_neighbors(plan_, (const double*)pos_.get(), n_, d_rcuts ? 0.0 : c.rcut, d_rcuts));
        surface_ = true;
        cache_valid_ = false;
    }
    bool surface() const { return surface_; }

    // host copy of the plan's neighbour list (after a surface assembly it
    // holds the accumulated lists)
    void refresh_list() {
        int64_t nn = 0, nnz = 0;
        check(dcpse_plan_info(plan_, &nn, &nnz, nullptr, nullptr, nullptr));
        const int64_t* drp = nullptr;
        const int32_t* dcl = nullptr;
        check(dcpse_neighbors_ptr(plan_, &drp, &dcl));
        rowptr_.resize((std::size_t)nn + 1);
        cols_.resize((std::size_t)nnz);
        check(dcpse_copy(rowptr_.data(), drp, (std::size_t)(nn + 1) * sizeof(int64_t)));
        if (nnz > 0) check(dcpse_copy(cols_.data(), dcl, (std::size_t)nnz * sizeof(int32_t)));
    }

    // Dcpse::p2p of term t: f is [n_support][ncomp], out [n][ncomp]
    void p2p(int t, const double* f, int ncomp, double* out) {
        fd_.upload(f, (std::size_t)std::max<int64_t>(n_sup_ * ncomp, 1) * sizeof(double));
        od_.ensure((std::size_t)std::max<int64_t>(n_ * ncomp, 1) * sizeof(double));
        check(dcpse_p2p_f64(plan_, t, (const double*)fd_.get(), ncomp, (double*)od_.get()));
        od_.download(out, (std::size_t)(n_ * ncomp) * sizeof(double));
    }
    int64_t n_support() const { return n_sup_; }
    void apply_term(int t, const double* f, double* out) {
        fd_.upload(f, (std::size_t)n_ * sizeof(double));
        od_.ensure((std::size_t)std::max<int64_t>(n_, 1) * sizeof(double));
        check(dcpse_apply_term_f64(plan_, t, (const double*)fd_.get(), (double*)od_.get()));
        od_.download(out, (std::size_t)n_ * sizeof(double));
    }

    // host copies of the kernels of every term, eps and eps^-|alpha|
    void fetch() {
        if (cache_valid_) return;
        const int T = n_terms();
        K_.assign(T, {});
        eip_.assign(T, {});
        eps_.assign((std::size_t)n_, 0.0);
        const double* de = nullptr;
        const int32_t* ds = nullptr;
        check(dcpse_eps_ptr(plan_, &de, &ds));
        if (n_ > 0) check(dcpse_copy(eps_.data(), de, (std::size_t)n_ * sizeof(double)));
        for (int t = 0; t < T; ++t) {
            const double *dk = nullptr, *dip = nullptr;
            check(dcpse_term_kernels_ptr(plan_, t, &dk, &dip));
            K_[t].assign((std::size_t)nnz(), 0.0);
            eip_[t].assign((std::size_t)n_, 0.0);
            if (nnz() > 0) check(dcpse_copy(K_[t].data(), dk, (std::size_t)nnz() * sizeof(double)));
            if (n_ > 0) check(dcpse_copy(eip_[t].data(), dip, (std::size_t)n_ * sizeof(double)));
        }
        cache_valid_ = true;
    }
    const std::vector<double>& kernels(int t) {
        fetch();
        return K_[t];
    }
    const std::vector<double>& eps_inv_pow(int t) {
        fetch();
        return eip_[t];
    }
    const std::vector<double>& eps() {
        fetch();
        return eps_;
    }
    void install(int t, const std::vector<double>& K, const std::vector<double>& eps, const std::vector<double>& eip) {
        DevBuf dk, de, di;
        dk.upload(K.data(), std::max<std::size_t>(K.size(), 1) * sizeof(double));
        de.upload(eps.data(), std::max<std::size_t>(eps.size(), 1) * sizeof(double));
        di.upload(eip.data(), std::max<std::size_t>(eip.size(), 1) * sizeof(double));
        check(dcpse_set_term_kernels(plan_, t, (const double*)dk.get(), (const double*)de.get(),
                                     (const double*)di.get()));
        cache_valid_ = false;
    }
    std::vector<std::vector<unsigned>> basis(int t) const {
        unsigned e[64 * 3];
        int nb = 0;
        check(dcpse_term_basis(plan_, t, e, 64, &nb));
        std::vector<std::vector<unsigned>> out(nb, std::vector<unsigned>(dim_));
        for (int i = 0; i < nb; ++i)
            for (int d = 0; d < dim_; ++d) out[i][d] = e[i * dim_ + d];
        return out;
    }

private:
    int dim_ = 0, nout_ = 0;
    dcpse_plan_t* plan_ = nullptr;
    int64_t n_ = 0, n_sup_ = 0;
    std::vector<unsigned> term_order_;
    std::vector<int64_t> rowptr_;
    std::vector<int32_t> cols_;
    DevBuf pos_, spos_, nrm_, spc_, rcs_, fd_, od_;
    PinBuf pin_f_, pin_o_;
    bool surface_ = false;
    bool cache_valid_ = false;
    std::vector<std::vector<double>> K_, eip_;
    std::vector<double> eps_;
    int last_fail_code_ = 0;
};

// Byte layout of Dcpse::save (Dcpse.hpp:302-331): openfpm's Packer writes
// each openfpm::vector of a primitive type as its element count (size_t)
// followed by the elements in native byte order, here localEps,
// localEpsInvPow, calcKernels (doubles) and kerOffsets (size_t), into
// file + "_" + rank.
template <typename T>
void pack_vector(std::ostream& out, const std::vector<T>& v) {
    const uint64_t n = (uint64_t)v.size();
    out.write((const char*)&n, sizeof n);
    out.write((const char*)v.data(), (std::streamsize)(v.size() * sizeof(T)));
}

template <typename T>
bool unpack_vector(std::istream& in, std::vector<T>& v, uint64_t max_elems) {
    uint64_t n = 0;
    in.read((char*)&n, sizeof n);
    if (!in || n > max_elems) return false;
    v.resize((std::size_t)n);
    in.read((char*)v.data(), (std::streamsize)(n * sizeof(T)));
    return (bool)in;
}

struct KernelSet {
    std::vector<double> eps, eip, K;
    std::vector<uint64_t> offsets;
};

inline bool write_kernel_file(const std::string& path, const KernelSet& k) {
    std::ofstream dump(path, std::ios::out | std::ios::binary);
    if (!dump.is_open()) return false;
    pack_vector(dump, k.eps);
    pack_vector(dump, k.eip);
    pack_vector(dump, k.K);
    pack_vector(dump, k.offsets);
    return (bool)dump;
}

inline bool read_kernel_file(const std::string& path, KernelSet& k) {
    std::ifstream in(path, std::ios::in | std::ios::binary | std::ios::ate);
    if (!in.is_open()) return false;
    const uint64_t bytes = (uint64_t)in.tellg();
    in.seekg(0);
    const uint64_t cap = bytes / sizeof(double);
    return unpack_vector(in, k.eps, cap) && unpack_vector(in, k.eip, cap) && unpack_vector(in, k.K, cap) &&
           unpack_vector(in, k.offsets, cap);
}

template <typename Sig>
std::vector<unsigned> sig_vector(const Sig& s, int dim) {
    std::vector<unsigned> v(dim);
    for (int d = 0; d < dim; ++d) v[d] = (unsigned)s.get(d);
    return v;
}

// D = sum_j (f_j + fxp) * K_j in the reference's order with every product
// and sum rounded separately (no contraction into fused multiply-adds, which
// compilers apply by default on some hosts), then D * eip.
#if defined(__clang__)
#define OPENFPM_DCPSE_NO_CONTRACT
#elif defined(__GNUC__)
#define OPENFPM_DCPSE_NO_CONTRACT __attribute__((optimize("fp-contract=off")))
#else
#define OPENFPM_DCPSE_NO_CONTRACT
#endif
template <typename T, typename FQ>
OPENFPM_DCPSE_NO_CONTRACT T reference_sum(std::size_t k, FQ fq, T fxp, const double* K, double eip) {
#if defined(__clang__)
#pragma clang fp contract(off)
#endif
    T D = 0;
    for (std::size_t j = 0; j < k; ++j) {
        const T t = fq(j) + fxp;
        const T prod = t * (T)K[j];
        D = D + prod;
    }
    return D * (T)eip;
}

// Neighbour lists built on the GPU: rows are the particles at dom, columns
// the particles at sup (or dom itself, with or without the particle in its
// own list when sup is null).
inline VerletList build_verlet(int dim, const std::vector<double>& dom, const std::vector<double>* sup, double rCut,
                               bool skip_ref, const std::vector<double>* rcut_pp = nullptr) {
    std::vector<unsigned> sig(dim, 0);
    sig[0] = 1;
    int terms = 1;
    dcpse_plan_t* plan = nullptr;
    check(dcpse_plan_create(&plan, dim, 1, &terms, sig.data(), 2, 0.9));
    std::unique_ptr<dcpse_plan_t, int (*)(dcpse_plan_t*)> guard(plan, dcpse_plan_destroy);
    const int64_t n = (int64_t)(dom.size() / dim);
    DevBuf dpos, spos;
    dpos.upload(dom.data(), std::max<std::size_t>(dom.size(), 1) * sizeof(double));
    if (sup) {
        spos.upload(sup->data(), std::max<std::size_t>(sup->size(), 1) * sizeof(double));
        check(dcpse_plan_set_support(plan, (const double*)spos.get(), (int64_t)(sup->size() / dim), 1));
    } else {
        check(dcpse_plan_set_support(plan, nullptr, 0, skip_ref ? 1 : 0));
    }
    DevBuf drc;
    if (rcut_pp) drc.upload(rcut_pp->data(), std::max<std::size_t>(rcut_pp->size(), 1) * sizeof(double));
    check(dcpse_build_neighbors(plan, (const double*)dpos.get(), n, rCut,
                                rcut_pp ? (const double*)drc.get() : nullptr));
    VerletList vl;
    vl.rCut = rCut;
    vl.skip_ref = skip_ref && !sup;
    if (rcut_pp) vl.rcuts = *rcut_pp;
    int64_t nn = 0, nnz = 0;
    check(dcpse_plan_info(plan, &nn, &nnz, nullptr, nullptr, nullptr));
    const int64_t* drp = nullptr;
    const int32_t* dcl = nullptr;
    check(dcpse_neighbors_ptr(plan, &drp, &dcl));
    vl.rowptr.resize((std::size_t)n + 1);
    vl.cols.resize((std::size_t)nnz);
    check(dcpse_copy(vl.rowptr.data(), drp, (std::size_t)(n + 1) * sizeof(int64_t)));
    if (nnz > 0) check(dcpse_copy(vl.cols.data(), dcl, (std::size_t)nnz * sizeof(int32_t)));
    return vl;
}

template <typename Parts>
std::vector<double> positions(Parts& parts, int dim) {
    const std::size_t n = parts.size_local();
    std::vector<double> pos(n * dim);
    for (std::size_t p = 0; p < n; ++p)
        for (int d = 0; d < dim; ++d) pos[p * dim + d] = (double)parts.getPos(p)[d];
    return pos;
}

inline void throw_too_few(int code, int64_t nbad) {
    if (nbad == 0) return;
    if (code == DCPSE_PART_TOO_FEW)
        throw std::length_error("Not enough neighbour points passed for Vandermonde matrix construction!");
    throw std::runtime_error("DC-PSE assembly failed for " + std::to_string(nbad) + " particle(s)");
}

}  // namespace detail

template <unsigned int dim, typename VerletList_type, typename vector_type, typename vector_type2 = vector_type>
class Dcpse {
public:
    typedef typename vector_type::stype T;
    typedef vector_type vtype;

    // c = HOverEpsilon: eps = <h> / c, <h> the mean L1 spacing of the support
    // (Dcpse.hpp:80; read at construction and at update)
    T HOverEpsilon = 0.9;

    virtual ~Dcpse() = default;

    template <typename Sig>
    Dcpse(vector_type& particles, VerletList_type& verletList, const Sig& differentialSignature,
          unsigned int convergenceOrder, T rCut, support_options opt = support_options::RADIUS)
        : verletList_(verletList),
          sig_(detail::sig_vector(differentialSignature, dim)),
          convergenceOrder_(convergenceOrder),
          rCut_(rCut),
          opt_(opt) {
        differentialOrder_ = 0;
        for (unsigned s : sig_) differentialOrder_ += s;
        support_ = &particles;
        domain_ = same_set(particles);
        particles.ghost_get_subset();
        plan_.reset(new detail::PlanHost(dim, {{sig_}}, convergenceOrder, (double)HOverEpsilon));
        plan_->set_particles(particles, verletList_);
        if (opt == support_options::LOAD) return;  // empty operator: load() or update later (Dcpse.hpp:703-707)
        assemble();
    }

    // Two particle sets (Dcpse.hpp:113-131): kernels of the domain particles
    // over supports drawn from particlesSupport (verletList rows = domain
    // particles, entries = support particles), as PPInterpolation uses.
    template <typename Sig>
    Dcpse(vector_type& particlesSupport, vector_type2& particlesDomain, VerletList_type& verletList,
          const Sig& differentialSignature, unsigned int convergenceOrder, T rCut,
          support_options opt = support_options::RADIUS)
        : verletList_(verletList),
          sig_(detail::sig_vector(differentialSignature, dim)),
          convergenceOrder_(convergenceOrder),
          rCut_(rCut),
          opt_(opt) {
        differentialOrder_ = 0;
        for (unsigned s : sig_) differentialOrder_ += s;
        support_ = &particlesSupport;
        domain_ = &particlesDomain;
        particlesSupport.ghost_get_subset();
        plan_.reset(new detail::PlanHost(dim, {{sig_}}, convergenceOrder, (double)HOverEpsilon));
        set_sets();
        if (opt == support_options::LOAD) return;
        assemble();
    }

protected:
    // Dcpse_gpu (below): eps = <h> / h_over_eps with the class's own factor
    template <typename Sig>
    Dcpse(vector_type& particles, VerletList_type& verletList, const Sig& differentialSignature,
          unsigned int convergenceOrder, T rCut, support_options opt, double h_over_eps)
        : HOverEpsilon((T)h_over_eps),
          verletList_(verletList),
          sig_(detail::sig_vector(differentialSignature, dim)),
          convergenceOrder_(convergenceOrder),
          rCut_(rCut),
          opt_(opt) {
        differentialOrder_ = 0;
        for (unsigned s : sig_) differentialOrder_ += s;
        support_ = &particles;
        domain_ = same_set(particles);
        particles.ghost_get_subset();
        plan_.reset(new detail::PlanHost(dim, {{sig_}}, convergenceOrder, (double)HOverEpsilon));
        plan_->set_particles(particles, verletList_);
        if (opt == support_options::LOAD) return;
        assemble();
    }

    // surface operators (SurfaceDcpse below)
    template <typename Sig>
    Dcpse(vector_type& particlesSupport, vector_type2& particlesDomain, VerletList_type& verletList,
          const Sig& differentialSignature, unsigned int convergenceOrder, T rCut, support_options opt,
          const detail::SurfaceCfg& surface)
        : verletList_(verletList),
          sig_(detail::sig_vector(differentialSignature, dim)),
          convergenceOrder_(convergenceOrder),
          rCut_(rCut),
          opt_(opt),
          surface_(surface) {
        differentialOrder_ = 0;
        for (unsigned s : sig_) differentialOrder_ += s;
        support_ = &particlesSupport;
        domain_ = &particlesDomain;
        plan_.reset(new detail::PlanHost(dim, {{sig_}}, convergenceOrder, (double)HOverEpsilon));
        set_sets();
        if (opt == support_options::LOAD) return;
        assemble();
    }

public:
    // Particle to particle interpolation (Dcpse.hpp:198-227): property prp2
    // of every domain particle = epsInvPow_p * sum_q f_q K_pq, f = property
    // prp1 of the support particles.
    template <unsigned int prp1, unsigned int prp2>
    void p2p() {
        const int64_t ns = plan_->n_support(), n = plan_->n();
        detail::check_rows(support_->size_local(), ns);
        detail::check_rows(domain_->size_local(), n);
        std::vector<double> f((std::size_t)ns), out((std::size_t)n);
        for (int64_t q = 0; q < ns; ++q) f[(std::size_t)q] = (double)support_->template getProp<prp1>(q);
        plan_->p2p(0, f.data(), 1, out.data());
        typedef typename std::remove_reference<decltype(domain_->template getProp<prp2>(0))>::type T2;
        for (int64_t p = 0; p < n; ++p) domain_->template getProp<prp2>(p) = (T2)out[(std::size_t)p];
    }

    // vector properties of N1 components (Dcpse.hpp:239-297)
    template <unsigned int prp1, unsigned int prp2, std::size_t N1>
    void p2p() {
        const int64_t ns = plan_->n_support(), n = plan_->n();
        detail::check_rows(support_->size_local(), ns);
        detail::check_rows(domain_->size_local(), n);
        std::vector<double> f((std::size_t)ns * N1), out((std::size_t)n * N1);
        for (int64_t q = 0; q < ns; ++q)
            for (std::size_t c = 0; c < N1; ++c)
                f[(std::size_t)q * N1 + c] = (double)support_->template getProp<prp1>(q)[c];
        plan_->p2p(0, f.data(), (int)N1, out.data());
        typedef typename std::remove_reference<decltype(domain_->template getProp<prp2>(0)[0])>::type T2;
        for (int64_t p = 0; p < n; ++p)
            for (std::size_t c = 0; c < N1; ++c)
                domain_->template getProp<prp2>(p)[c] = (T2)out[(std::size_t)p * N1 + c];
    }

    // Bulk apply: Df at every particle from property fValuePos into
    // DfValuePos (Dcpse.hpp:467-499).
    template <unsigned int fValuePos, unsigned int DfValuePos>
    void computeDifferentialOperator(vector_type& particles) {
        const int64_t n = plan_->n();
        std::vector<double> f((std::size_t)n), out((std::size_t)n);
        for (int64_t p = 0; p < n; ++p) f[(std::size_t)p] = (double)particles.template getProp<fValuePos>(p);
        plan_->apply_term(0, f.data(), out.data());
        for (int64_t p = 0; p < n; ++p) particles.template getProp<DfValuePos>(p) = (T)out[(std::size_t)p];
    }

    // Per-key form (Dcpse.hpp:560-603): o1.value(key) gives the field.
    template <typename op_type>
    T computeDifferentialOperator(const vect_dist_key_dx& p, op_type& o1) {
        const auto& K = plan_->kernels(0);
        const auto& eip = plan_->eps_inv_pow(0);
        const T sign = (differentialOrder_ % 2 == 0) ? -1 : 1;
        const T fxp = sign * o1.value(p);
        const int64_t b = plan_->rowptr()[p.getKey()];
        const std::size_t k = verletList_.getNNPart(p.getKey());
        auto fq = [&](std::size_t j) -> T {
            return o1.value(vect_dist_key_dx(verletList_.get(p.getKey(), j)));
        };
        return detail::reference_sum<T>(k, fq, fxp, K.data() + b, eip[p.getKey()]);
    }

    // accessors (Dcpse.hpp:507-550)
    int getNumNN(const vect_dist_key_dx& p) { return (int)verletList_.getNNPart(p.getKey()); }
    T getCoeffNN(const vect_dist_key_dx& p, int j) {
        return plan_->kernels(0)[(std::size_t)(plan_->rowptr()[p.getKey()] + j)];
    }
    std::size_t getIndexNN(const vect_dist_key_dx& p, int q) { return verletList_.get(p.getKey(), q); }
    T getSign() { return (differentialOrder_ % 2 == 0 && differentialOrder_ != 0) ? -1 : 1; }
    T getEpsilonInvPrefactor(const vect_dist_key_dx& p) { return plan_->eps_inv_pow(0)[p.getKey()]; }

    // after particles moved (and the Verlet list was updated): Dcpse.hpp:675-687
    void initializeUpdate(vector_type& particles) {
        support_ = &particles;
        domain_ = same_set(particles);
        plan_.reset(new detail::PlanHost(dim, {{sig_}}, convergenceOrder_, (double)HOverEpsilon));
        if (surface_.on) {
            surface_.refresh();
            set_sets();
        } else {
            plan_->set_particles(particles, verletList_);
        }
        assemble();
    }
    void initializeUpdate(vector_type& particlesSupport, vector_type2& particlesDomain) {
        support_ = &particlesSupport;
        domain_ = &particlesDomain;
        plan_.reset(new detail::PlanHost(dim, {{sig_}}, convergenceOrder_, (double)HOverEpsilon));
        if (surface_.on) surface_.refresh();
        set_sets();
        assemble();
    }

    // Dcpse::save (Dcpse.hpp:302-331): localEps, localEpsInvPow, calcKernels
    // and kerOffsets in openfpm's Packer layout, to file + "_" + rank (rank 0)
    void save(const std::string& file) {
        detail::KernelSet k;
        k.eps = plan_->eps();
        k.eip = plan_->eps_inv_pow(0);
        k.K = plan_->kernels(0);
        k.offsets.assign(plan_->rowptr().begin(), plan_->rowptr().end() - (plan_->n() > 0 ? 1 : 0));
        if (!detail::write_kernel_file(file + "_0", k))
            std::cerr << __FILE__ << ":" << __LINE__ << " Unable to write " << file << "_0" << std::endl;
    }

    // Dcpse::load (Dcpse.hpp:337-379): the neighbour list of the constructor
    // must be the one the file was saved with (checked through kerOffsets)
    void load(const std::string& file) {
        detail::KernelSet k;
        if (!detail::read_kernel_file(file + "_0", k)) {
            std::cerr << __FILE__ << ":" << __LINE__ << " error, opening file: " << file << std::endl;
            return;
        }
        if ((int64_t)k.eps.size() != plan_->n() || k.eip.size() != k.eps.size() ||
            (int64_t)k.K.size() != plan_->nnz() || k.offsets.size() != k.eps.size() ||
            !std::equal(k.offsets.begin(), k.offsets.end(), plan_->rowptr().begin(),
                        [](uint64_t a, int64_t b) { return (int64_t)a == b; })) {
            std::cerr << __FILE__ << ":" << __LINE__ << " error, " << file << " does not match this operator"
                      << std::endl;
            return;
        }
        plan_->install(0, k.K, k.eps, k.eip);
    }

    // min / max over particles of each moment sum_q K_pq m_j(x_pq / eps_p)
    // (Dcpse.hpp:381-457)
    void checkMomenta(vector_type& particles) {
        const auto B = plan_->basis(0);
        const auto& K = plan_->kernels(0);
        const auto& eps = plan_->eps();
        std::vector<double> mn(B.size(), 3000000000.0), mx(B.size(), -3000000000.0);
        for (int64_t p = 0; p < plan_->n(); ++p) {
            std::vector<double> acc(B.size(), 0.0);
            const int64_t b = plan_->rowptr()[p];
            for (int64_t j = b; j < plan_->rowptr()[p + 1]; ++j) {
                const std::size_t q = (std::size_t)plan_->cols()[j];
                for (std::size_t i = 0; i < B.size(); ++i) {
                    double m = 1.0;
                    for (int d = 0; d < (int)dim; ++d)
                        m *= std::pow(((double)particles.getPos(p)[d] - (double)particles.getPos(q)[d]) / eps[p],
                                      (double)B[i][d]);
                    acc[i] += m * K[j];
                }
            }
            for (std::size_t i = 0; i < B.size(); ++i) {
                mn[i] = std::min(mn[i], acc[i]);
                mx[i] = std::max(mx[i], acc[i]);
            }
        }
        for (std::size_t i = 0; i < B.size(); ++i) {
            std::cout << "MOMENTA: 1 :";
            for (int d = 0; d < (int)dim; ++d) std::cout << " " << B[i][d];
            std::cout << " Min: " << mn[i] << "  Max: " << mx[i] << std::endl;
        }
    }

    // adds the kernel of particle p to property prp of its neighbours (Dcpse.hpp:151-163)
    template <unsigned int prp>
    void DrawKernel(vector_type& particles, int p) {
        const auto& K = plan_->kernels(0);
        const int64_t b = plan_->rowptr()[p];
        for (int64_t j = b; j < plan_->rowptr()[p + 1]; ++j)
            particles.template getProp<prp>((std::size_t)plan_->cols()[j]) += K[j];
    }

    dcpse_plan_t* plan() const { return plan_->plan(); }

private:
    void assemble() {
        int64_t nbad = plan_->assemble(DCPSE_STORE_TERMS_F64);
        detail::throw_too_few(plan_->last_fail_code(), nbad);
        // a surface operator replaces the caller's lists with the
        // accumulated ones, as the reference does (Dcpse.hpp:1001-1005)
        if constexpr (std::is_same<VerletList_type, VerletList>::value)
            if (surface_.on) {
                verletList_.rowptr = plan_->rowptr();
                verletList_.cols = plan_->cols();
            }
    }

    // the domain set of a one-set operator is the support set itself
    vector_type2* same_set(vector_type& particles) {
        if constexpr (std::is_same<vector_type, vector_type2>::value)
            return &particles;
        else
            return nullptr;
    }

    // one set when both references name the same object
    void set_sets() {
        const bool two = (const void*)support_ != (const void*)domain_;
        if (surface_.on)
            plan_->set_surface_particles(*support_, *domain_, two, surface_);
        else
            plan_->set_particles(*support_, *domain_, verletList_, two);
    }

    vector_type* support_ = nullptr;
    vector_type2* domain_ = nullptr;
    VerletList_type& verletList_;
    std::vector<unsigned> sig_;
    unsigned differentialOrder_ = 0;
    unsigned convergenceOrder_;
    T rCut_;
    support_options opt_;
    detail::SurfaceCfg surface_;
    std::unique_ptr<detail::PlanHost> plan_;
};

namespace detail {
// the support list a Dcpse_gpu builds for itself (held in a base class so it
// exists before the Dcpse base that refers to it)
struct OwnSupport {
    VerletList own_support;
    OwnSupport(int dim, const std::vector<double>& pos, double rCut)
        : own_support(build_verlet(dim, pos, nullptr, rCut, true)) {}
};
}  // namespace detail

// Dcpse_gpu (Dcpse.cuh:35-875), the class behind the reference's *_gpu
// operators.  What it computes differs from Dcpse in two points, both kept:
// eps = 2 <h> (FACTOR = 2, Dcpse.cuh:799-807; no HOverEpsilon), and the
// support is built by the class from rCut (SupportBuilderGPU,
// SupportBuilder.cuh:14-107: |x_p - x_q| < rCut, p excluded), the Verlet list
// argument being unused as there.  The reference solves the moment systems
// by an unpivoted batched LU; here they go through the same column-pivoting
// QR as Dcpse, which gives the same kernels up to the systems' conditioning.
template <unsigned int dim, typename VerletList_type, typename vector_type>
class Dcpse_gpu : private detail::OwnSupport, public Dcpse<dim, VerletList, vector_type> {
    typedef Dcpse<dim, VerletList, vector_type> base;

public:
    typedef typename vector_type::stype T;

    template <typename Sig>
    Dcpse_gpu(vector_type& particles, VerletList_type& verletList, const Sig& differentialSignature,
              unsigned int convergenceOrder, T rCut, support_options opt = support_options::RADIUS)
        : detail::OwnSupport(dim, detail::positions(particles, dim), (double)rCut),
          base(particles, own_support, differentialSignature, convergenceOrder, rCut, opt, 0.5),
          rCutGpu_((double)rCut) {
        (void)verletList;
    }

    // the support is rebuilt from the moved particles before re-assembly
    void initializeUpdate(vector_type& particles) {
        own_support = detail::build_verlet(dim, detail::positions(particles, dim), nullptr, rCutGpu_, true);
        base::initializeUpdate(particles);
    }

private:
    double rCutGpu_;
};

// SurfaceDcpse (Dcpse.hpp:829-1085): the support of every particle is
// extended by nCount virtual particles on each side along the normal
// (property NORMAL_ID of the support set), the kernels are assembled on the
// extended support and every virtual particle's kernel is added onto its
// surface particle.  The Verlet list handed in gives the cutoff and whether
// a particle is its own neighbour, and receives the accumulated lists.
// support_options::ADAPTIVE takes the spacing along the normal per particle
// from property 0 / nCount and the cutoffs of an adaptive Verlet list
// (getVerletAdaptRCut), as the reference does (Dcpse.hpp:1055-1066, 881-909).
template <unsigned int dim, typename VerletList_type, typename vector_type, typename vector_type2 = vector_type>
class SurfaceDcpse : public Dcpse<dim, VerletList_type, vector_type, vector_type2> {
    typedef Dcpse<dim, VerletList_type, vector_type, vector_type2> base;

public:
    template <typename Sig, unsigned int NORMAL_ID>
    SurfaceDcpse(vector_type& particlesSupport, vector_type2& particlesDomain, VerletList_type& verletList,
                 const Sig& differentialSignature, unsigned int convergenceOrder, typename base::T rCut,
                 typename base::T nSpacing, unsigned int nCount, value_t<NORMAL_ID>,
                 support_options opt = support_options::RADIUS)
        : base(particlesSupport, particlesDomain, verletList, differentialSignature, convergenceOrder, rCut, opt,
               detail::surface_cfg<NORMAL_ID>(particlesSupport, verletList, (double)rCut, (double)nSpacing, nCount,
                                              opt)) {}
};

}  // namespace openfpm_dcpse
