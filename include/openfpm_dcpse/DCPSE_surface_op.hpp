// DCPSE_surface_op.hpp -- drop-in for openfpm_numerics' surface DC-PSE
// operators (src/DCPSE/DCPSE_op/DCPSE_surface_op.hpp) on the GB300 C-ABI:
//     SurfaceDerivative_xx<NORMAL_ID, VerletList_type> op(parts, verletList, ord, rCut, nSpacing, nCount);
//     getV<0>(parts) = op(getV<3>(parts)) + ...;
// NORMAL_ID names the property holding the unit normals.  Each operator is a
// SurfaceDcpse of one signature: the support is extended along the normals,
// assembled on the GPU and accumulated back onto the surface particles; the
// Verlet list passed in gives the cutoff and receives the accumulated lists.
#pragma once

#include "DCPSE_op.hpp"

namespace openfpm_dcpse {

template <unsigned int NORMAL_ID, typename VerletList_type>
class SurfaceOperator : public DcpseOperator<VerletList_type> {
public:
    template <typename particles_type>
    SurfaceOperator(particles_type& parts, VerletList_type& verletList, unsigned int ord,
                    typename particles_type::stype rCut, typename particles_type::stype nSpacing, unsigned int nCount,
                    std::vector<unsigned> sig, support_options opt)
        : DcpseOperator<VerletList_type>(parts, verletList, ord, {{sig}}, opt,
                                         detail::surface_cfg<NORMAL_ID>(parts, verletList, (double)rCut,
                                                                        (double)nSpacing, nCount, opt)) {}
};

#define OPENFPM_DCPSE_SURFACE_OP(NAME, SIGEXPR)                                                                 \
    template <unsigned int NORMAL_ID, typename VerletList_type>                                                \
    class NAME : public SurfaceOperator<NORMAL_ID, VerletList_type> {                                          \
    public:                                                                                                    \
        template <typename particles_type>                                                                     \
        NAME(particles_type& parts, VerletList_type& verletList, unsigned int ord,                             \
             typename particles_type::stype rCut, typename particles_type::stype nSpacing, unsigned int nCount, \
             support_options opt = support_options::RADIUS)                                                     \
            : SurfaceOperator<NORMAL_ID, VerletList_type>(                                                      \
                  parts, verletList, ord, rCut, nSpacing, nCount,                                               \
                  [](int dim) { return SIGEXPR; }(particles_type::dims), opt) {}                                \
    };

// DCPSE_surface_op.hpp:11-1020
OPENFPM_DCPSE_SURFACE_OP(SurfaceDerivative_x, detail::unit(dim, 0))
OPENFPM_DCPSE_SURFACE_OP(SurfaceDerivative_y, detail::unit(dim, 1))
OPENFPM_DCPSE_SURFACE_OP(SurfaceDerivative_z, detail::unit(dim, 2))
OPENFPM_DCPSE_SURFACE_OP(SurfaceDerivative_xx, detail::unit(dim, 0, 2))
OPENFPM_DCPSE_SURFACE_OP(SurfaceDerivative_yy, detail::unit(dim, 1, 2))
OPENFPM_DCPSE_SURFACE_OP(SurfaceDerivative_zz, detail::unit(dim, 2, 2))
OPENFPM_DCPSE_SURFACE_OP(SurfaceDerivative_xy, detail::mixed(dim, {{0, 1}, {1, 1}}))
OPENFPM_DCPSE_SURFACE_OP(SurfaceDerivative_yz, detail::mixed(dim, {{1, 1}, {2, 1}}))
OPENFPM_DCPSE_SURFACE_OP(SurfaceDerivative_xz, detail::mixed(dim, {{0, 1}, {2, 1}}))
// the reference builds Laplace_Beltrami as one Dcpse of signature (2, 2, 2)
// (DCPSE_surface_op.hpp:326-347), kept as is
OPENFPM_DCPSE_SURFACE_OP(Laplace_Beltrami, std::vector<unsigned>(dim, 2))
#undef OPENFPM_DCPSE_SURFACE_OP

// SurfaceDerivative_G (DCPSE_surface_op.hpp:1022-1100): signature p
template <unsigned int NORMAL_ID, typename VerletList_type>
class SurfaceDerivative_G : public SurfaceOperator<NORMAL_ID, VerletList_type> {
public:
    template <typename particles_type, typename Sig>
    SurfaceDerivative_G(particles_type& parts, VerletList_type& verletList, unsigned int ord,
                        typename particles_type::stype rCut, typename particles_type::stype nSpacing,
                        unsigned int nCount, const Sig& p, support_options opt = support_options::RADIUS)
        : SurfaceOperator<NORMAL_ID, VerletList_type>(parts, verletList, ord, rCut, nSpacing, nCount,
                                                      detail::sig_vector(p, particles_type::dims), opt) {}
};

}  // namespace openfpm_dcpse
