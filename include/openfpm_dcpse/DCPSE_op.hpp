// DCPSE_op.hpp -- drop-in for openfpm_numerics' DC-PSE operator classes
// (src/DCPSE/DCPSE_op/DCPSE_op.hpp): Derivative_x/y/z, Derivative_xx/yy/zz,
// Derivative_xy/yz/xz, the third and fourth order ones, Derivative_G,
// Laplacian and Gradient, with the same constructors
//     Op<VerletList_type> op(parts, verletList, ord, rCut [, opt])
// and the same use in assignments
//     getV<1>(parts) = Lap(getV<0>(parts));
//     getV<1>(parts) = 2 * Dx(getV<0>(parts)) + Dy(getV<0>(parts));
// Each operator owns one GB300 plan holding all of its reference Dcpse terms
// (a Laplacian's dim terms 2e_i share one neighbour list and one moment
// matrix); an assignment evaluates every operator node on the GPU in FP64 in
// the reference's order (VECT_DCPSE :65-67, VECT_DCPSE_V :144-153,
// VECT_DCPSE_V_SUM :388-399) and combines the nodes on the host.
// Divergence, Advection and Curl2D are operator nodes too.  Only linear
// combinations of operator nodes are supported on the right-hand side (the
// reference's general expression engine is not part of this path).
#pragma once

#include <algorithm>
#include <array>
#include <functional>
#include <memory>
#include <stdexcept>
#include <string>
#include <tuple>
#include <type_traits>
#include <vector>

#include "Dcpse.hpp"

namespace openfpm_dcpse {

const double dcpse_oversampling_factor = 1.9;  // DCPSE_op.hpp:20
const double rcut_verlet = 3.1;                // DCPSE_op.hpp:21

// ------------------------------------------------------------ expressions --
template <unsigned int prp, typename vector_type>
struct PropRef;

// One operator applied to one property: result[c][p] for c < ncomp.
struct Node {
    std::function<void(std::vector<std::vector<double>>&)> eval;
    int ncomp = 1;
    double coef = 1.0;
};

struct Expr {
    std::vector<Node> nodes;
};

inline Expr operator*(double c, Expr e) {
    for (auto& n : e.nodes) n.coef *= c;
    return e;
}
inline Expr operator*(Expr e, double c) { return c * e; }
inline Expr operator+(Expr a, const Expr& b) {
    a.nodes.insert(a.nodes.end(), b.nodes.begin(), b.nodes.end());
    return a;
}
inline Expr operator-(Expr a, Expr b) { return a + (-1.0) * b; }

namespace detail {
template <typename V>
auto prop_component(V& v, int c, std::true_type) -> decltype(v[c])& {
    return v[c];
}
template <typename V>
V& prop_component(V& v, int, std::false_type) {
    return v;
}
template <typename V, typename = void>
struct is_indexable : std::false_type {};
template <typename V>
struct is_indexable<V, std::void_t<decltype(std::declval<V&>()[0])>> : std::true_type {};

// components of a property: N for std::array<T, N> or T[N], else 1
template <typename V, typename = void>
struct prop_ncomp : std::integral_constant<int, 1> {};
template <typename V>
struct prop_ncomp<V, std::enable_if_t<(std::tuple_size<V>::value > 0)>>
    : std::integral_constant<int, (int)std::tuple_size<V>::value> {};
template <typename T, std::size_t N>
struct prop_ncomp<T[N], void> : std::integral_constant<int, (int)N> {};
}  // namespace detail

// getV<prp>(parts): a property of a particle set, usable as an operand and
// as the target of an assignment.
template <unsigned int prp, typename vector_type>
struct PropRef {
    vector_type& v;
    typedef vector_type vtype;
    vector_type& getVector() const { return v; }

    typedef typename std::remove_reference<decltype(std::declval<vector_type&>().template getProp<prp>(0))>::type
        prop_type;
    static constexpr int ncomp = detail::prop_ncomp<prop_type>::value;

    std::vector<double> values() const { return component(0); }

    // component c of every particle (the value itself for a scalar property)
    std::vector<double> component(int c) const {
        std::vector<double> f(v.size_local());
        for (std::size_t p = 0; p < f.size(); ++p)
            f[p] = (double)detail::prop_component(v.template getProp<prp>(p), c, detail::is_indexable<prop_type>{});
        return f;
    }

    // getV<prp>(parts) = expr: evaluate every node and combine
    PropRef& operator=(const Expr& e) {
        const std::size_t n = v.size_local();
        int ncomp = e.nodes.empty() ? 1 : e.nodes[0].ncomp;
        typedef typename std::remove_reference<decltype(v.template getProp<prp>(0))>::type PT;
        std::vector<std::vector<double>> tmp;
        if (e.nodes.size() == 1 && e.nodes[0].coef == 1.0) {
            // one operator: its result goes straight into the property
            e.nodes[0].eval(tmp);
            for (std::size_t p = 0; p < n; ++p)
                for (int c = 0; c < ncomp; ++c)
                    detail::prop_component(v.template getProp<prp>(p), c, detail::is_indexable<PT>{}) = tmp[c][p];
            return *this;
        }
        std::vector<std::vector<double>> acc(ncomp, std::vector<double>(n, 0.0));
        bool first = true;
        for (const auto& node : e.nodes) {
            if (node.ncomp != ncomp) throw std::invalid_argument("mixing scalar and vector operator results");
            node.eval(tmp);
            for (int c = 0; c < ncomp; ++c)
                for (std::size_t p = 0; p < n; ++p)
                    acc[c][p] = (first && node.coef == 1.0) ? tmp[c][p] : acc[c][p] + node.coef * tmp[c][p];
            first = false;
        }
        for (std::size_t p = 0; p < n; ++p)
            for (int c = 0; c < ncomp; ++c) {
                auto& slot = detail::prop_component(v.template getProp<prp>(p), c, detail::is_indexable<PT>{});
                slot = acc[c][p];
            }
        return *this;
    }
};

template <unsigned int prp, typename vector_type>
PropRef<prp, vector_type> getV(vector_type& v) {
    return PropRef<prp, vector_type>{v};
}

// Verlet list of a particle set built on the GPU: every q with
// |x_p - x_q|^2 < rCut^2 in ascending q, without q == p unless skip_ref is
// false (the roles of vector_dist::getVerlet<VL_NON_SYMMETRIC|VL_SKIP_REF_PART>
// and getVerlet<VL_NON_SYMMETRIC>).
template <typename particles_type>
VerletList getVerlet(particles_type& parts, double rCut, bool skip_ref = true) {
    const int dim = particles_type::dims;
    return detail::build_verlet(dim, detail::positions(parts, dim), nullptr, rCut, skip_ref);
}

// vector_dist::getVerletAdaptRCut: every particle's cutoff is its property
// 0; q is a neighbour of p when |x_p - x_q|^2 < rCut_p^2
template <typename particles_type>
VerletList getVerletAdaptRCut(particles_type& parts, bool skip_ref = true) {
    const int dim = particles_type::dims;
    std::vector<double> rc(parts.size_local());
    for (std::size_t p = 0; p < parts.size_local(); ++p) rc[p] = (double)parts.template getProp<0>(p);
    return detail::build_verlet(dim, detail::positions(parts, dim), nullptr, 0.0, skip_ref, &rc);
}

// --------------------------------------------------------------- operators --
// Which reference class an operator's terms follow: Dcpse (the default), or
// Dcpse_gpu for the *_gpu aliases (DCPSE_op.hpp:3510-3530), i.e. eps = 2 <h>
// and a support the operator builds from rCut itself (see Dcpse_gpu).
struct dcpse_cpu_kind {
    static constexpr bool gpu = false;
};
struct dcpse_gpu_kind {
    static constexpr bool gpu = true;
};

// outputs: list of outputs, each a list of signatures summed into it.
template <typename VerletList_type, typename Kind = dcpse_cpu_kind>
class DcpseOperator {
public:
    template <typename particles_type>
    DcpseOperator(particles_type& parts, VerletList_type& verletList, unsigned int ord,
                  typename particles_type::stype rCut, std::vector<std::vector<std::vector<unsigned>>> outputs,
                  support_options opt, double h_over_eps = 0.9)
        : vl_(verletList),
          outputs_(std::move(outputs)),
          ord_(ord),
          hoe_(Kind::gpu ? 0.5 : h_over_eps),
          dim_(particles_type::dims),
          rcut_((double)rCut) {
        parts.ghost_get_subset();
        build(parts, opt != support_options::LOAD);
    }

    // initializeUpdate of every Dcpse term (DCPSE_op.hpp:779-785); a surface
    // operator extends the support again from the current normals
    template <typename particles_type>
    void update(particles_type& parts) {
        if (surf_.on) surf_.refresh();
        build(parts, true);
    }

    template <typename particles_type>
    void deallocate(particles_type&) {
        plan_.reset();
    }

    // operand: getV<i>(parts).  By default every output is the reference's
    // own sum of its Dcpse terms in FP64, in the reference's order (one pass
    // per term).  After set_apply_precision(DCPSE_F32 / DCPSE_F32_RESID /
    // DCPSE_F32_BUDGET / DCPSE_F32_PAIR) all outputs come from one batched pass over the
    // summed weights (see dcpse_capi.h), through pinned staging buffers.
    template <unsigned int prp, typename vector_type>
    Expr operator()(PropRef<prp, vector_type> arg) {
        Node nd;
        nd.ncomp = (int)outputs_.size();
        detail::PlanHost* P = plan_.get();
        const std::size_t outs = outputs_.size();
        const int prec = precision_;
        nd.eval = [P, arg, outs, prec](std::vector<std::vector<double>>& out) {
            std::vector<double> f = arg.values();
            detail::check_rows(f.size(), P->n());
            if (prec != DCPSE_F64) {
                P->apply_batched(prec, f.data(), out);
                return;
            }
            out.assign(outs, std::vector<double>(f.size()));
            for (std::size_t o = 0; o < outs; ++o) P->apply_output((int)o, f.data(), out[o].data());
        };
        Expr e;
        e.nodes.push_back(nd);
        return e;
    }

    // Precision of the expression applies (no counterpart in the reference,
    // whose operators apply in FP64 only): DCPSE_F64 (default), DCPSE_F32,
    // DCPSE_F32_RESID or DCPSE_F32_BUDGET (with the plan's error budget,
    // 1e-6 unless set_error_budget says otherwise).  Re-assembles when the
    // weights it needs are not stored yet.
    void set_apply_precision(int precision) {
        int flags = DCPSE_STORE_TERMS_F64 | DCPSE_STORE_OUT_F32;
        if (precision == DCPSE_F32_RESID) flags |= DCPSE_STORE_OUT_F32_RESID;
        if (precision == DCPSE_F32_BUDGET || precision == DCPSE_F32_PAIR) flags |= DCPSE_STORE_OUT_F32_CORR;
        if (precision != DCPSE_F64 && precision != DCPSE_F32 && precision != DCPSE_F32_RESID &&
            precision != DCPSE_F32_BUDGET && precision != DCPSE_F32_PAIR)
            throw std::invalid_argument("DC-PSE operator: unknown precision");
        if ((flags | asm_flags_) != asm_flags_) {
            asm_flags_ |= flags;
            int64_t nbad = plan_->assemble(asm_flags_);
            detail::throw_too_few(plan_->last_fail_code(), nbad);
        }
        precision_ = precision;
    }
    void set_error_budget(double budget) { detail::check(dcpse_plan_set_error_budget(plan_->plan(), budget, DCPSE_F32)); }

    // FP32 batched apply of every output of this operator (one pass)
    template <unsigned int prp, typename vector_type>
    std::vector<std::vector<double>> apply_f32(PropRef<prp, vector_type> arg) {
        std::vector<double> f = arg.values();
        detail::check_rows(f.size(), plan_->n());
        std::vector<double> flat(outputs_.size() * f.size());
        detail::check(dcpse_apply_batched_host(plan_->plan(), f.data(), flat.data(), DCPSE_F32));
        std::vector<std::vector<double>> out(outputs_.size());
        for (std::size_t o = 0; o < outputs_.size(); ++o)
            out[o].assign(flat.begin() + o * f.size(), flat.begin() + (o + 1) * f.size());
        return out;
    }

    template <typename particles_type>
    void save(particles_type&, const std::string& file) {
        save_impl(file);
    }
    template <typename particles_type>
    void load(particles_type&, const std::string& file) {
        load_impl(file);
    }

    // adds the kernels (all terms) of particle k to property prp of its neighbours
    template <unsigned int prp, typename particles_type>
    void DrawKernel(particles_type& particles, int k) {
        for (int t = 0; t < plan_->n_terms(); ++t) {
            const auto& K = plan_->kernels(t);
            for (int64_t j = plan_->rowptr()[k]; j < plan_->rowptr()[k + 1]; ++j)
                particles.template getProp<prp>((std::size_t)plan_->cols()[j]) += K[j];
        }
    }

    dcpse_plan_t* plan() const { return plan_->plan(); }

protected:
    detail::PlanHost* host() const { return plan_.get(); }

    // surface operators (DCPSE_surface_op.hpp)
    template <typename particles_type>
    DcpseOperator(particles_type& parts, VerletList_type& verletList, unsigned int ord,
                  std::vector<std::vector<std::vector<unsigned>>> outputs, support_options opt,
                  const detail::SurfaceCfg& surf)
        : vl_(verletList), outputs_(std::move(outputs)), ord_(ord), hoe_(0.9), dim_(particles_type::dims),
          surf_(surf) {
        build(parts, opt != support_options::LOAD);
    }

private:
    template <typename particles_type>
    void build(particles_type& parts, bool assemble) {
        plan_.reset(new detail::PlanHost(dim_, outputs_, ord_, hoe_));
        if (surf_.on) {
            plan_->set_surface_particles(parts, parts, false, surf_);
        } else if constexpr (Kind::gpu) {
            own_vl_ = getVerlet(parts, rcut_);
            plan_->set_particles(parts, own_vl_);
        } else {
            plan_->set_particles(parts, vl_);
        }
        if (!assemble) return;
        int64_t nbad = plan_->assemble(asm_flags_);
        detail::throw_too_few(plan_->last_fail_code(), nbad);
        // a surface operator hands the accumulated lists back (Dcpse.hpp:1001-1005)
        if constexpr (std::is_same<VerletList_type, VerletList>::value)
            if (surf_.on) {
                vl_.rowptr = plan_->rowptr();
                vl_.cols = plan_->cols();
            }
    }

    // one Dcpse file per term in Dcpse::save's layout: file + "_0" for an
    // operator of one term (what the reference's Derivative_* save writes),
    // file + "_term<t>_0" for each term of a sum or vector operator
    std::string term_file(const std::string& file, int t) const {
        return plan_->n_terms() == 1 ? file + "_0" : file + "_term" + std::to_string(t) + "_0";
    }
    void save_impl(const std::string& file) {
        for (int t = 0; t < plan_->n_terms(); ++t) {
            detail::KernelSet k;
            k.eps = plan_->eps();
            k.eip = plan_->eps_inv_pow(t);
            k.K = plan_->kernels(t);
            k.offsets.assign(plan_->rowptr().begin(), plan_->rowptr().end() - (plan_->n() > 0 ? 1 : 0));
            if (!detail::write_kernel_file(term_file(file, t), k)) {
                std::cerr << __FILE__ << ":" << __LINE__ << " Unable to write " << term_file(file, t) << std::endl;
                return;
            }
        }
    }
    void load_impl(const std::string& file) {
        std::vector<detail::KernelSet> ks((std::size_t)plan_->n_terms());
        for (int t = 0; t < plan_->n_terms(); ++t) {
            detail::KernelSet& k = ks[(std::size_t)t];
            if (!detail::read_kernel_file(term_file(file, t), k)) {
                std::cerr << __FILE__ << ":" << __LINE__ << " error, opening file: " << term_file(file, t) << std::endl;
                return;
            }
            if ((int64_t)k.eps.size() != plan_->n() || k.eip.size() != k.eps.size() ||
                (int64_t)k.K.size() != plan_->nnz() || k.offsets.size() != k.eps.size() ||
                !std::equal(k.offsets.begin(), k.offsets.end(), plan_->rowptr().begin(),
                            [](uint64_t a, int64_t b) { return (int64_t)a == b; })) {
                std::cerr << __FILE__ << ":" << __LINE__ << " error, " << term_file(file, t)
                          << " does not match this operator" << std::endl;
                return;
            }
        }
        for (int t = 0; t < plan_->n_terms(); ++t)
            plan_->install(t, ks[(std::size_t)t].K, ks[(std::size_t)t].eps, ks[(std::size_t)t].eip);
    }

    VerletList_type& vl_;
    std::vector<std::vector<std::vector<unsigned>>> outputs_;
    unsigned ord_;
    double hoe_;
    int dim_;
    double rcut_ = 0.0;
    int precision_ = DCPSE_F64;
    int asm_flags_ = DCPSE_STORE_TERMS_F64 | DCPSE_STORE_OUT_F32;
    VerletList own_vl_;  // the support of a Dcpse_gpu-kind operator
    detail::SurfaceCfg surf_;
    std::unique_ptr<detail::PlanHost> plan_;
};

namespace detail {
inline std::vector<unsigned> unit(int dim, int axis, unsigned power = 1) {
    std::vector<unsigned> s(dim, 0);
    s[axis] = power;
    return s;
}
inline std::vector<unsigned> mixed(int dim, std::initializer_list<std::pair<int, unsigned>> l) {
    std::vector<unsigned> s(dim, 0);
    for (auto& p : l) s[p.first] = p.second;
    return s;
}
}  // namespace detail

#define OPENFPM_DCPSE_SINGLE_OP(NAME, SIGEXPR)                                                                  \
    template <typename VerletList_type, typename Kind = dcpse_cpu_kind>                                        \
    class NAME : public DcpseOperator<VerletList_type, Kind> {                                                 \
    public:                                                                                                    \
        template <typename particles_type>                                                                     \
        NAME(particles_type& parts, VerletList_type& verletList, unsigned int ord,                             \
             typename particles_type::stype rCut, support_options opt = support_options::RADIUS)               \
            : DcpseOperator<VerletList_type, Kind>(parts, verletList, ord, rCut,                               \
                                             {{[](int dim) { return SIGEXPR; }(particles_type::dims)}}, opt) {} \
    };

// Derivative_x_T ... (DCPSE_op.hpp:649-3385)
OPENFPM_DCPSE_SINGLE_OP(Derivative_x, detail::unit(dim, 0))
OPENFPM_DCPSE_SINGLE_OP(Derivative_y, detail::unit(dim, 1))
OPENFPM_DCPSE_SINGLE_OP(Derivative_z, detail::unit(dim, 2))
OPENFPM_DCPSE_SINGLE_OP(Derivative_xx, detail::unit(dim, 0, 2))
OPENFPM_DCPSE_SINGLE_OP(Derivative_yy, detail::unit(dim, 1, 2))
OPENFPM_DCPSE_SINGLE_OP(Derivative_zz, detail::unit(dim, 2, 2))
OPENFPM_DCPSE_SINGLE_OP(Derivative_xy, detail::mixed(dim, {{0, 1}, {1, 1}}))
OPENFPM_DCPSE_SINGLE_OP(Derivative_yz, detail::mixed(dim, {{1, 1}, {2, 1}}))
OPENFPM_DCPSE_SINGLE_OP(Derivative_xz, detail::mixed(dim, {{0, 1}, {2, 1}}))
OPENFPM_DCPSE_SINGLE_OP(Derivative_xxx, detail::unit(dim, 0, 3))
OPENFPM_DCPSE_SINGLE_OP(Derivative_yyy, detail::unit(dim, 1, 3))
OPENFPM_DCPSE_SINGLE_OP(Derivative_xxy, detail::mixed(dim, {{0, 2}, {1, 1}}))
OPENFPM_DCPSE_SINGLE_OP(Derivative_yyx, detail::mixed(dim, {{0, 1}, {1, 2}}))
OPENFPM_DCPSE_SINGLE_OP(Derivative_xxxx, detail::unit(dim, 0, 4))
OPENFPM_DCPSE_SINGLE_OP(Derivative_yyyy, detail::unit(dim, 1, 4))
OPENFPM_DCPSE_SINGLE_OP(Derivative_xxyy, detail::mixed(dim, {{0, 2}, {1, 2}}))
#undef OPENFPM_DCPSE_SINGLE_OP

// Derivative_G_T (DCPSE_op.hpp:3387-3482): arbitrary signature p
template <typename VerletList_type, typename Kind = dcpse_cpu_kind>
class Derivative_G : public DcpseOperator<VerletList_type, Kind> {
public:
    template <typename particles_type, typename Sig>
    Derivative_G(particles_type& parts, VerletList_type& verletList, unsigned int ord,
                 typename particles_type::stype rCut, const Sig& p, support_options opt = support_options::RADIUS)
        : DcpseOperator<VerletList_type, Kind>(parts, verletList, ord, rCut,
                                         {{detail::sig_vector(p, particles_type::dims)}}, opt) {}
};

// Laplacian_T (DCPSE_op.hpp:1350-1500): one output, sum of dim terms 2e_i
template <typename VerletList_type, typename Kind = dcpse_cpu_kind>
class Laplacian : public DcpseOperator<VerletList_type, Kind> {
    static std::vector<std::vector<std::vector<unsigned>>> outs(int dim) {
        std::vector<std::vector<unsigned>> t;
        for (int i = 0; i < dim; ++i) t.push_back(detail::unit(dim, i, 2));
        return {t};
    }

public:
    template <typename particles_type>
    Laplacian(particles_type& parts, VerletList_type& verletList, unsigned int ord, typename particles_type::stype rCut,
              support_options opt = support_options::RADIUS)
        : DcpseOperator<VerletList_type, Kind>(parts, verletList, ord, rCut, outs(particles_type::dims), opt) {}
};

// Gradient_T (DCPSE_op.hpp:1081-1224): dim outputs e_i (vector result)
template <typename VerletList_type, typename Kind = dcpse_cpu_kind>
class Gradient : public DcpseOperator<VerletList_type, Kind> {
    static std::vector<std::vector<std::vector<unsigned>>> outs(int dim) {
        std::vector<std::vector<std::vector<unsigned>>> o;
        for (int i = 0; i < dim; ++i) o.push_back({detail::unit(dim, i)});
        return o;
    }

public:
    template <typename particles_type>
    Gradient(particles_type& parts, VerletList_type& verletList, unsigned int ord, typename particles_type::stype rCut,
             support_options opt = support_options::RADIUS)
        : DcpseOperator<VerletList_type, Kind>(parts, verletList, ord, rCut, outs(particles_type::dims), opt) {}
};

// Divergence_T (DCPSE_op.hpp:1503-1630): dim terms e_i applied to the
// components of a vector property, VECT_DCPSE_V_DIV (:446-475):
// div = ((0 + D_0 v_0) + D_1 v_1) + ...
template <typename VerletList_type, typename Kind = dcpse_cpu_kind>
class Divergence : public DcpseOperator<VerletList_type, Kind> {
    static std::vector<std::vector<std::vector<unsigned>>> outs(int dim) {
        std::vector<std::vector<std::vector<unsigned>>> o;
        for (int i = 0; i < dim; ++i) o.push_back({detail::unit(dim, i)});
        return o;
    }

public:
    template <typename particles_type>
    Divergence(particles_type& parts, VerletList_type& verletList, unsigned int ord,
               typename particles_type::stype rCut, support_options opt = support_options::RADIUS)
        : DcpseOperator<VerletList_type, Kind>(parts, verletList, ord, rCut, outs(particles_type::dims), opt),
          dim_(particles_type::dims) {}

    template <unsigned int prp, typename vector_type>
    Expr operator()(PropRef<prp, vector_type> arg) {
        Node nd;
        nd.ncomp = 1;
        detail::PlanHost* P = this->host();
        const int dim = dim_;
        nd.eval = [P, arg, dim](std::vector<std::vector<double>>& out) {
            const std::size_t n = arg.v.size_local();
            detail::check_rows(n, P->n());
            out.assign(1, std::vector<double>(n, 0.0));
            std::vector<double> d(n);
            for (int i = 0; i < dim; ++i) {
                std::vector<double> f = arg.component(i);
                P->apply_output(i, f.data(), d.data());
                for (std::size_t p = 0; p < n; ++p) out[0][p] = out[0][p] + d[p];
            }
        };
        Expr e;
        e.nodes.push_back(nd);
        return e;
    }

private:
    int dim_;
};

// Advection_T (DCPSE_op.hpp:1632-1781): (v . grad) f, VECT_DCPSE_V_DOT
// (:531-565): adv = ((0 + v_0 D_0 f) + v_1 D_1 f) + ..., component-wise for a
// vector property f
template <typename VerletList_type, typename Kind = dcpse_cpu_kind>
class Advection : public Divergence<VerletList_type, Kind> {
public:
    using Divergence<VerletList_type, Kind>::Divergence;

    template <unsigned int p1, typename vt1, unsigned int p2, typename vt2>
    Expr operator()(PropRef<p1, vt1> vel, PropRef<p2, vt2> arg) {
        Node nd;
        nd.ncomp = PropRef<p2, vt2>::ncomp;
        detail::PlanHost* P = this->host();
        const int dim = vt1::dims;
        nd.eval = [P, vel, arg, dim](std::vector<std::vector<double>>& out) {
            const std::size_t n = arg.v.size_local();
            detail::check_rows(n, P->n());
            detail::check_rows(vel.v.size_local(), P->n());
            const int nc = PropRef<p2, vt2>::ncomp;
            out.assign(nc, std::vector<double>(n, 0.0));
            std::vector<double> d(n);
            for (int c = 0; c < nc; ++c) {
                std::vector<double> f = arg.component(c);
                for (int i = 0; i < dim; ++i) {
                    const std::vector<double> vi = vel.component(i);
                    P->apply_output(i, f.data(), d.data());
                    for (std::size_t p = 0; p < n; ++p) out[c][p] = out[c][p] + vi[p] * d[p];
                }
            }
        };
        Expr e;
        e.nodes.push_back(nd);
        return e;
    }
};

// Curl2D_T (DCPSE_op.hpp:1227-1340): terms e_1 and e_0, VECT_DCPSE_V_CURL2D
// (:206-233): (D_y f, -D_x f)
template <typename VerletList_type, typename Kind = dcpse_cpu_kind>
class Curl2D : public DcpseOperator<VerletList_type, Kind> {
    static std::vector<std::vector<std::vector<unsigned>>> outs(int dim) {
        return {{detail::unit(dim, 1)}, {detail::unit(dim, 0)}};
    }

public:
    template <typename particles_type>
    Curl2D(particles_type& parts, VerletList_type& verletList, unsigned int ord, typename particles_type::stype rCut,
           support_options opt = support_options::RADIUS)
        : DcpseOperator<VerletList_type, Kind>(parts, verletList, ord, rCut, outs(particles_type::dims), opt) {}

    template <unsigned int prp, typename vector_type>
    Expr operator()(PropRef<prp, vector_type> arg) {
        Expr e = DcpseOperator<VerletList_type, Kind>::operator()(arg);
        auto inner = e.nodes[0].eval;
        e.nodes[0].eval = [inner](std::vector<std::vector<double>>& out) {
            inner(out);
            for (auto& x : out[1]) x = -x;
        };
        return e;
    }
};

// GPU aliases of the reference (DCPSE_op.hpp:3510-3530): the same operators
// over Dcpse_gpu (eps = 2 <h>, support built from rCut)
template <typename VL> using Derivative_x_gpu = Derivative_x<VL, dcpse_gpu_kind>;
template <typename VL> using Derivative_y_gpu = Derivative_y<VL, dcpse_gpu_kind>;
template <typename VL> using Derivative_z_gpu = Derivative_z<VL, dcpse_gpu_kind>;
template <typename VL> using Derivative_xx_gpu = Derivative_xx<VL, dcpse_gpu_kind>;
template <typename VL> using Derivative_yy_gpu = Derivative_yy<VL, dcpse_gpu_kind>;
template <typename VL> using Derivative_zz_gpu = Derivative_zz<VL, dcpse_gpu_kind>;
template <typename VL> using Derivative_xy_gpu = Derivative_xy<VL, dcpse_gpu_kind>;
template <typename VL> using Laplacian_gpu = Laplacian<VL, dcpse_gpu_kind>;
template <typename VL> using Gradient_gpu = Gradient<VL, dcpse_gpu_kind>;
template <typename VL> using Derivative_G_gpu = Derivative_G<VL, dcpse_gpu_kind>;
template <typename VL> using Derivative_yz_gpu = Derivative_yz<VL, dcpse_gpu_kind>;
template <typename VL> using Derivative_xz_gpu = Derivative_xz<VL, dcpse_gpu_kind>;
template <typename VL> using Derivative_xxx_gpu = Derivative_xxx<VL, dcpse_gpu_kind>;
template <typename VL> using Derivative_xxy_gpu = Derivative_xxy<VL, dcpse_gpu_kind>;
template <typename VL> using Derivative_yyx_gpu = Derivative_yyx<VL, dcpse_gpu_kind>;
template <typename VL> using Derivative_yyy_gpu = Derivative_yyy<VL, dcpse_gpu_kind>;
template <typename VL> using Divergence_gpu = Divergence<VL, dcpse_gpu_kind>;
template <typename VL> using Advection_gpu = Advection<VL, dcpse_gpu_kind>;
template <typename VL> using Curl2D_gpu = Curl2D<VL, dcpse_gpu_kind>;

}  // namespace openfpm_dcpse
