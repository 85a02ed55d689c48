// particles.hpp -- minimal stand-ins for the openfpm types the DC-PSE API
// touches (Point, vector_dist, VerletList, vect_dist_key_dx), for code that
// uses the GB300 DC-PSE headers without openfpm_data / openfpm_pdata.
//
// Dcpse and the operator classes are templates over the particle and list
// types and only call the members below, so openfpm's own vector_dist and
// VerletList work in their place:
//   particles: size_local(), getPos(key)[d] (or .get(d)), getProp<i>(key)
//   list:      getNNPart(p), get(p, j)
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <initializer_list>
#include <stdexcept>
#include <tuple>
#include <vector>

namespace openfpm_dcpse {

template <unsigned int dim, typename T>
struct Point {
    std::array<T, dim> v{};
    Point() = default;
    Point(std::initializer_list<T> l) {
        std::size_t i = 0;
        for (T x : l)
            if (i < dim) v[i++] = x;
    }
    T& get(unsigned i) { return v[i]; }
    const T& get(unsigned i) const { return v[i]; }
    T& operator[](unsigned i) { return v[i]; }
    const T& operator[](unsigned i) const { return v[i]; }
    void zero() { v.fill(T(0)); }
    const T* asArray() const { return v.data(); }
};

// key of a particle (vect_dist_key_dx in openfpm)
struct vect_dist_key_dx {
    std::size_t k = 0;
    vect_dist_key_dx() = default;
    explicit vect_dist_key_dx(std::size_t key) : k(key) {}
    std::size_t getKey() const { return k; }
};

// Particle set: positions and a tuple of per-particle properties
// (aggregate<T0, T1, ...> in openfpm).
template <unsigned int dims_, typename stype_, typename... Props>
class vector_dist {
public:
    static constexpr unsigned int dims = dims_;
    typedef stype_ stype;

    explicit vector_dist(std::size_t n = 0) { resize(n); }

    void resize(std::size_t n) {
        pos_.assign(n * dims, stype(0));
        std::apply([n](auto&... v) { (v.assign(n, {}), ...); }, props_);
    }
    void add() { resize(size_local() + 1); }
    std::size_t size_local() const { return pos_.size() / dims; }
    std::size_t size_local_with_ghost() const { return size_local(); }

    stype* getPos(std::size_t p) { return &pos_[p * dims]; }
    const stype* getPos(std::size_t p) const { return &pos_[p * dims]; }
    stype* getPos(vect_dist_key_dx p) { return getPos(p.getKey()); }
    stype* getLastPos() { return getPos(size_local() - 1); }

    template <unsigned int i>
    auto& getProp(std::size_t p) {
        return std::get<i>(props_)[p];
    }
    template <unsigned int i>
    auto& getProp(vect_dist_key_dx p) {
        return std::get<i>(props_)[p.getKey()];
    }
    template <unsigned int i>
    auto& getLastProp() {
        return std::get<i>(props_)[size_local() - 1];
    }
    template <unsigned int i>
    auto* propData() {
        return std::get<i>(props_).data();
    }
    stype* posData() { return pos_.data(); }

    // no ghosts on a single GPU: minimum-image offsets handle periodicity
    void ghost_get_subset() {}
    template <unsigned int... i>
    void ghost_get() {}
    void map() {}

private:
    std::vector<stype> pos_;
    std::tuple<std::vector<Props>...> props_;
};

// CSR Verlet list (VL_NON_SYMMETRIC | VL_SKIP_REF_PART semantics): every
// q != p with |x_p - x_q|^2 < rCut^2, ascending q.
class VerletList {
public:
    std::vector<int64_t> rowptr{0};
    std::vector<int32_t> cols;
    double rCut = 0.0;        // cutoff the list was built with
    bool skip_ref = true;     // VL_SKIP_REF_PART: a particle is not its own neighbour
    std::vector<double> rcuts;  // per-particle cutoffs of an adaptive list (empty: rCut for all)

    double getRCuts(std::size_t p) const { return rcuts.empty() ? rCut : rcuts[p]; }

    std::size_t getNNPart(std::size_t p) const { return (std::size_t)(rowptr[p + 1] - rowptr[p]); }
    std::size_t getNNPart(vect_dist_key_dx p) const { return getNNPart(p.getKey()); }
    std::size_t get(std::size_t p, std::size_t j) const { return (std::size_t)cols[rowptr[p] + j]; }
    std::size_t get(vect_dist_key_dx p, std::size_t j) const { return get(p.getKey(), j); }
    std::size_t size() const { return rowptr.size() - 1; }
};

// openfpm's value_t<i>: a tag naming property i (here the property that
// holds the unit normals of a surface operator)
template <unsigned int i>
struct value_t {};

}  // namespace openfpm_dcpse
