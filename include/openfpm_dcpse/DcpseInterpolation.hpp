// DcpseInterpolation.hpp -- drop-in for openfpm_numerics' PPInterpolation
// (src/DCPSE/DcpseInterpolation.hpp:28-195) on the GB300 C-ABI.
//
//     auto vl = createVerletTwoPhase(domain, support, rCut);
//     PPInterpolation<Support, Domain, VerletList> Fx(support, domain, vl, 2, rCut);
//     Fx.p2p<0, 1>();          // domain prop 1 = interpolation of support prop 0
//     Fx.p2p<2, 3, 3>();       // vector properties of 3 components
//
// The operator is a Dcpse with the zero signature on two particle sets
// (Dcpse.hpp:113-131); p2p evaluates epsInvPow_p * sum_q f_q K_pq on the GPU
// in the reference's operation order (dcpse_p2p_f64).  The surface form
// (the constructor taking nSpacing and isSurfaceInterpolation) builds a
// SurfaceDcpse over the support set extended along its normals (property
// NORMAL_ID) with nCount = rCut / nSpacing virtual particles per side.
#pragma once

#include <climits>

#include "Dcpse.hpp"

namespace openfpm_dcpse {

// Lists of the support particles within rCut of every domain particle
// (openfpm's createVerletTwoPhase, DCPSE_op_test_base_tests.cpp:369-372).
// The reference also takes the support set's cell list; the lists here are
// built on the GPU, so it is not needed.
template <typename domain_type, typename support_type>
VerletList createVerletTwoPhase(domain_type& particlesDomain, support_type& particlesSupport, double rCut) {
    const int dim = domain_type::dims;
    const std::vector<double> sup = detail::positions(particlesSupport, dim);
    return detail::build_verlet(dim, detail::positions(particlesDomain, dim), &sup, rCut, false);
}

template <typename domain_type, typename support_type, typename cell_list_type>
VerletList createVerletTwoPhase(domain_type& particlesDomain, support_type& particlesSupport, cell_list_type&,
                                double rCut) {
    return createVerletTwoPhase(particlesDomain, particlesSupport, rCut);
}

template <typename particlesSupport_type, typename particlesDomain_type, typename VerletList_type,
          std::size_t NORMAL_ID = INT_MAX>
class PPInterpolation {
    typedef Dcpse<particlesSupport_type::dims, VerletList_type, particlesSupport_type, particlesDomain_type> dcpse_type;

public:
    PPInterpolation(particlesSupport_type& particlesSupport, particlesDomain_type& particlesDomain,
                    VerletList_type& verletList, unsigned int ord, typename particlesSupport_type::stype rCut,
                    support_options opt = support_options::RADIUS)
        : particlesSupport_(particlesSupport), particlesDomain_(particlesDomain) {
        Point<particlesSupport_type::dims, unsigned int> p;
        p.zero();
        dcpse_ = new dcpse_type(particlesSupport, particlesDomain, verletList, p, ord, rCut, opt);
    }

    // surface interpolation (DcpseInterpolation.hpp:94-113)
    PPInterpolation(particlesSupport_type& particlesSupport, particlesDomain_type& particlesDomain,
                    VerletList_type& verletList, unsigned int ord, typename particlesSupport_type::stype rCut,
                    typename particlesSupport_type::stype nSpacing, bool isSurfaceInterpolation,
                    support_options opt = support_options::RADIUS)
        : particlesSupport_(particlesSupport), particlesDomain_(particlesDomain) {
        Point<particlesSupport_type::dims, unsigned int> p;
        p.zero();
        if (!isSurfaceInterpolation) {
            dcpse_ = new dcpse_type(particlesSupport, particlesDomain, verletList, p, ord, rCut, opt);
            return;
        }
        typedef SurfaceDcpse<particlesSupport_type::dims, VerletList_type, particlesSupport_type, particlesDomain_type>
            surface_type;
        dcpse_ = new surface_type(particlesSupport, particlesDomain, verletList, p, ord, rCut, nSpacing,
                                  static_cast<unsigned int>(rCut / nSpacing), value_t<NORMAL_ID>(), opt);
    }

    // p2p<propSupport, propDomain>() (DcpseInterpolation.hpp:133-137)
    template <unsigned int propSupport, unsigned int propDomain>
    void p2p() {
        dcpse_->template p2p<propSupport, propDomain>();
    }

    // vector properties of N1 components (DcpseInterpolation.hpp:150-154)
    template <unsigned int propSupport, unsigned int propDomain, std::size_t N1>
    void p2p() {
        dcpse_->template p2p<propSupport, propDomain, N1>();
    }

    // DcpseInterpolation.hpp:187-190
    void update() { dcpse_->initializeUpdate(particlesSupport_, particlesDomain_); }

    void deallocate() {
        delete dcpse_;
        dcpse_ = nullptr;
    }

    dcpse_type& dcpse() { return *dcpse_; }

private:
    dcpse_type* dcpse_ = nullptr;
    particlesSupport_type& particlesSupport_;
    particlesDomain_type& particlesDomain_;
};

}  // namespace openfpm_dcpse
