// Problem classes written against the ScaFES callback interface (test
// infrastructure for the drop-in Problem).  Each derives directly from
// ScaFES::Problem and restates one of the reference's system-test problems:
//   HeatLin    -- heat equation, Dirichlet border, exact solution
//                 (1+t)(1+x+y+z)  (tests/system/HeatEqnFDM/Dirichlet/TimeLinSpaceLin)
//   PennesLin  -- Pennes bioheat with perfusion, same exact solution
//                 (tests/system/PennesBioheatEqnFDM/Dirichlet/TimeLinSpaceLin)
//   MirrorPow2 -- the 2/7 averaging stencil with the mirrored border,
//                 exact solution 2^n (i+j+k) (tests/system/HeatEqnFdmStencilWidthOne)
//   HeatSine   -- heat equation, Dirichlet 0, u0 = sin(pi x) sin(pi y) sin(pi z)
//   HeatFlux<KIND> -- heat equation, Dirichlet at the min faces and a Neumann
//                 (KIND 0) or Cauchy (KIND 1) flux condition at the max faces,
//                 exact solution (1+t)(1+x+y+z)
//                 (tests/system/HeatEqnFDM/{Neumann,Cauchy}/TimeLinSpaceLin)
//   PennesRadiation -- Pennes bioheat, Dirichlet at the min faces and the
//                 radiation condition -lambda du/dn = eps sigma u^4 - G at the
//                 max faces, G quartic in time, exact solution (1+t)(1+x+y+z)
//                 (tests/system/PennesBioheatEqnFDM/Radiation/TimeLinSpaceLin)
//   TissueTumour -- Pennes bioheat whose perfusion and metabolic heat take
//                 another value inside a tumour sphere, Neumann faces and a
//                 convective (Cauchy) z-max face (examples/TumorHeatEqnFDM)
//   TissueMri  -- Pennes bioheat with every coefficient a known field over
//                 the nodes, Neumann faces, a closed-skull (Neumann) z-max
//                 face and convection + radiation where the "surface" field
//                 is 1 (examples/MRIDataPBHEqnFDM)
//   YeeCavity  -- Maxwell's equations in a perfectly conducting box on the
//                 staggered Yee grid (eps = mu = 1, cubic spacing): six
//                 unknown fields Ex Ey Ez Hx Hy Hz, the H half step in
//                 updateInner/updateBorder and the E step in the leapfrog
//                 second phase updateInner2/updateBorder2, as the reference's
//                 FDTD example splits them (examples/EMFDTD/EMFDTD.hpp:295-385,
//                 without its absorbing layers and source)
// The tissue classes evaluate their expressions in the examples' operation
// order, so that the recorded weights are the same doubles.
#pragma once

#include <cmath>
#include <vector>

#include "ScaFES.hpp"

template <typename CT, std::size_t DIM>
class HeatLin : public ScaFES::Problem<HeatLin<CT, DIM>, CT, DIM> {
    using Base = ScaFES::Problem<HeatLin<CT, DIM>, CT, DIM>;
public:
    using Base::Base;
    const double RHO = 1.0, C = 1.0, LAMBDA = 1.0;
    static double lin(const ScaFES::Ntuple<double, DIM>& x) {
        double s = 1.0;
        for (std::size_t p = 0; p < DIM; ++p) s += x[p];
        return s;
    }
    void evalInner(std::vector<ScaFES::DataField<CT, DIM>>& v, const ScaFES::Ntuple<int, DIM>& n, const int& t) {
        const double s = lin(this->coordinates(n));
        v[0](n) = s * (RHO * C);          // heat source f
        v[1](n) = 0.0;                    // border value g (unused inside)
        v[2](n) = s * (1.0 + this->time(t));  // exact solution
    }
    void evalBorder(std::vector<ScaFES::DataField<CT, DIM>>& v, const ScaFES::Ntuple<int, DIM>& n, const int& t) {
        const double s = lin(this->coordinates(n));
        v[0](n) = 0.0;
        v[1](n) = s * (1.0 + this->time(t));
        v[2](n) = v[1](n);
    }
    template <typename TT>
    void initInner(std::vector<ScaFES::DataField<TT, DIM>>& v, const std::vector<TT>&, const ScaFES::Ntuple<int, DIM>& n, const int& t) {
        v[0](n) = lin(this->coordinates(n)) * (1.0 + this->time(t));
    }
    template <typename TT>
    void initBorder(std::vector<ScaFES::DataField<TT, DIM>>& v, const std::vector<TT>& o, const ScaFES::Ntuple<int, DIM>& n, const int& t) {
        initInner<TT>(v, o, n, t);
    }
    template <typename TT>
    void updateInner(std::vector<ScaFES::DataField<TT, DIM>>& vNew, const std::vector<ScaFES::DataField<TT, DIM>>& vOld,
                     const ScaFES::Ntuple<int, DIM>& n, const int&) {
        vNew[0](n) = vOld[0](n);
        for (std::size_t p = 0; p < DIM; ++p)
            vNew[0](n) += this->tau() * (LAMBDA / (RHO * C)) *
                          (vOld[0](this->connect(n, 2 * p)) + vOld[0](this->connect(n, 2 * p + 1)) - 2.0 * vOld[0](n)) /
                          (this->gridsize(p) * this->gridsize(p));
        vNew[0](n) += this->tau() * (1.0 / (RHO * C)) * this->knownDfOld(0, n);
    }
    template <typename TT>
    void updateBorder(std::vector<ScaFES::DataField<TT, DIM>>& vNew, const std::vector<ScaFES::DataField<TT, DIM>>&,
                      const ScaFES::Ntuple<int, DIM>& n, const int&) {
        vNew[0](n) = this->knownDf(1, n);
    }
    template <typename TT>
    void updateInner2(std::vector<ScaFES::DataField<TT, DIM>>&, const std::vector<ScaFES::DataField<TT, DIM>>&, const ScaFES::Ntuple<int, DIM>&, const int&) {}
    template <typename TT>
    void updateBorder2(std::vector<ScaFES::DataField<TT, DIM>>&, const std::vector<ScaFES::DataField<TT, DIM>>&, const ScaFES::Ntuple<int, DIM>&, const int&) {}
    const std::vector<ScaFES::DataField<CT, DIM>>& latest() const { return this->mVectUnknownDfsDomOld; }
};

template <typename CT, std::size_t DIM>
class PennesLin : public ScaFES::Problem<PennesLin<CT, DIM>, CT, DIM> {
    using Base = ScaFES::Problem<PennesLin<CT, DIM>, CT, DIM>;
public:
    using Base::Base;
    const double RHO = 1.0, C = 1.0, LAMBDA = 1.0, RHO_B = 1.0, C_B = 1.0, W = 1.0;
    void evalInner(std::vector<ScaFES::DataField<CT, DIM>>& v, const ScaFES::Ntuple<int, DIM>& n, const int& t) {
        const double s = HeatLin<CT, DIM>::lin(this->coordinates(n));
        v[0](n) = s * (RHO * C) + RHO_B * C_B * W * (s * (1.0 + this->time(t)));
        v[1](n) = 0.0;
        v[2](n) = s * (1.0 + this->time(t));
    }
    void evalBorder(std::vector<ScaFES::DataField<CT, DIM>>& v, const ScaFES::Ntuple<int, DIM>& n, const int& t) {
        const double s = HeatLin<CT, DIM>::lin(this->coordinates(n));
        v[0](n) = 0.0;
        v[1](n) = s * (1.0 + this->time(t));
        v[2](n) = v[1](n);
    }
    template <typename TT>
    void initInner(std::vector<ScaFES::DataField<TT, DIM>>& v, const std::vector<TT>&, const ScaFES::Ntuple<int, DIM>& n, const int& t) {
        v[0](n) = HeatLin<CT, DIM>::lin(this->coordinates(n)) * (1.0 + this->time(t));
    }
    template <typename TT>
    void initBorder(std::vector<ScaFES::DataField<TT, DIM>>& v, const std::vector<TT>& o, const ScaFES::Ntuple<int, DIM>& n, const int& t) {
        initInner<TT>(v, o, n, t);
    }
    template <typename TT>
    void updateInner(std::vector<ScaFES::DataField<TT, DIM>>& vNew, const std::vector<ScaFES::DataField<TT, DIM>>& vOld,
                     const ScaFES::Ntuple<int, DIM>& n, const int&) {
        vNew[0](n) = vOld[0](n);
        for (std::size_t p = 0; p < DIM; ++p)
            vNew[0](n) += this->tau() * (LAMBDA / (RHO * C)) *
                          (vOld[0](this->connect(n, 2 * p)) + vOld[0](this->connect(n, 2 * p + 1)) - 2.0 * vOld[0](n)) /
                          (this->gridsize(p) * this->gridsize(p));
        vNew[0](n) -= this->tau() * ((RHO_B * C_B) / (RHO * C)) * W * vOld[0](n);
        vNew[0](n) += this->tau() * (1.0 / (RHO * C)) * this->knownDfOld(0, n);
    }
    template <typename TT>
    void updateBorder(std::vector<ScaFES::DataField<TT, DIM>>& vNew, const std::vector<ScaFES::DataField<TT, DIM>>&,
                      const ScaFES::Ntuple<int, DIM>& n, const int&) {
        vNew[0](n) = this->knownDf(1, n);
    }
    template <typename TT>
    void updateInner2(std::vector<ScaFES::DataField<TT, DIM>>&, const std::vector<ScaFES::DataField<TT, DIM>>&, const ScaFES::Ntuple<int, DIM>&, const int&) {}
    template <typename TT>
    void updateBorder2(std::vector<ScaFES::DataField<TT, DIM>>&, const std::vector<ScaFES::DataField<TT, DIM>>&, const ScaFES::Ntuple<int, DIM>&, const int&) {}
    const std::vector<ScaFES::DataField<CT, DIM>>& latest() const { return this->mVectUnknownDfsDomOld; }
};

template <typename CT, std::size_t DIM>
class MirrorPow2 : public ScaFES::Problem<MirrorPow2<CT, DIM>, CT, DIM> {
    using Base = ScaFES::Problem<MirrorPow2<CT, DIM>, CT, DIM>;
public:
    using Base::Base;
    void evalInner(std::vector<ScaFES::DataField<CT, DIM>>& v, const ScaFES::Ntuple<int, DIM>& n, const int& t) {
        double s = 0.0;
        for (std::size_t p = 0; p < DIM; ++p) s += n[p];
        v[0](n) = s * std::pow(2.0, t);
    }
    void evalBorder(std::vector<ScaFES::DataField<CT, DIM>>& v, const ScaFES::Ntuple<int, DIM>& n, const int& t) { evalInner(v, n, t); }
    template <typename TT>
    void initInner(std::vector<ScaFES::DataField<TT, DIM>>& v, const std::vector<TT>&, const ScaFES::Ntuple<int, DIM>& n, const int&) {
        v[0](n) = 0.0;
        for (std::size_t p = 0; p < DIM; ++p) v[0](n) += n[p];
    }
    template <typename TT>
    void initBorder(std::vector<ScaFES::DataField<TT, DIM>>& v, const std::vector<TT>& o, const ScaFES::Ntuple<int, DIM>& n, const int& t) {
        initInner<TT>(v, o, n, t);
    }
    template <typename TT>
    void updateInner(std::vector<ScaFES::DataField<TT, DIM>>& vNew, const std::vector<ScaFES::DataField<TT, DIM>>& vOld,
                     const ScaFES::Ntuple<int, DIM>& n, const int&) {
        vNew[0](n) = vOld[0](n);
        for (std::size_t d = 0; d < 2 * DIM; ++d) vNew[0](n) += vOld[0](this->connect(n, d));
        vNew[0](n) *= 2.0 / (2 * DIM + 1);
    }
    template <typename TT>
    void updateBorder(std::vector<ScaFES::DataField<TT, DIM>>& vNew, const std::vector<ScaFES::DataField<TT, DIM>>& vOld,
                      const ScaFES::Ntuple<int, DIM>& n, const int& t) {
        TT corr = std::pow(2.0, t - 1);
        for (std::size_t d = 0; d < 2 * DIM; ++d) {
            if (ScaFES::Ntuple<int, DIM>(-(int)(d + 1)) == this->connect(n, d)) {
                const int opp = (d % 2 == 0) ? (int)d + 1 : (int)d - 1;
                const double sgn = (d % 2 == 0) ? 1.0 : -1.0;
                vNew[0](n) = vOld[0](n) + vOld[0](this->connect(n, opp)) - sgn * corr;
            }
        }
    }
    template <typename TT>
    void updateInner2(std::vector<ScaFES::DataField<TT, DIM>>&, const std::vector<ScaFES::DataField<TT, DIM>>&, const ScaFES::Ntuple<int, DIM>&, const int&) {}
    template <typename TT>
    void updateBorder2(std::vector<ScaFES::DataField<TT, DIM>>&, const std::vector<ScaFES::DataField<TT, DIM>>&, const ScaFES::Ntuple<int, DIM>&, const int&) {}
    const std::vector<ScaFES::DataField<CT, DIM>>& latest() const { return this->mVectUnknownDfsDomOld; }
};

template <typename CT, std::size_t DIM>
class HeatSine : public ScaFES::Problem<HeatSine<CT, DIM>, CT, DIM> {
    using Base = ScaFES::Problem<HeatSine<CT, DIM>, CT, DIM>;
public:
    using Base::Base;
    void evalInner(std::vector<ScaFES::DataField<CT, DIM>>& v, const ScaFES::Ntuple<int, DIM>& n, const int&) {
        v[0](n) = 0.0;
        v[1](n) = 0.0;
    }
    void evalBorder(std::vector<ScaFES::DataField<CT, DIM>>& v, const ScaFES::Ntuple<int, DIM>& n, const int& t) { evalInner(v, n, t); }
    template <typename TT>
    void initInner(std::vector<ScaFES::DataField<TT, DIM>>& v, const std::vector<TT>&, const ScaFES::Ntuple<int, DIM>& n, const int&) {
        const ScaFES::Ntuple<double, DIM> x = this->coordinates(n);
        double s = 1.0;
        for (std::size_t p = 0; p < DIM; ++p) s *= std::sin(M_PI * x[p]);
        v[0](n) = s;
    }
    template <typename TT>
    void initBorder(std::vector<ScaFES::DataField<TT, DIM>>& v, const std::vector<TT>&, const ScaFES::Ntuple<int, DIM>& n, const int&) {
        v[0](n) = 0.0;
    }
    template <typename TT>
    void updateInner(std::vector<ScaFES::DataField<TT, DIM>>& vNew, const std::vector<ScaFES::DataField<TT, DIM>>& vOld,
                     const ScaFES::Ntuple<int, DIM>& n, const int&) {
        vNew[0](n) = vOld[0](n);
        for (std::size_t p = 0; p < DIM; ++p)
            vNew[0](n) += this->tau() * (vOld[0](this->connect(n, 2 * p)) + vOld[0](this->connect(n, 2 * p + 1)) - 2.0 * vOld[0](n)) /
                          (this->gridsize(p) * this->gridsize(p));
        vNew[0](n) += this->tau() * this->knownDfOld(0, n);
    }
    template <typename TT>
    void updateBorder(std::vector<ScaFES::DataField<TT, DIM>>& vNew, const std::vector<ScaFES::DataField<TT, DIM>>&,
                      const ScaFES::Ntuple<int, DIM>& n, const int&) {
        vNew[0](n) = this->knownDf(1, n);
    }
    template <typename TT>
    void updateInner2(std::vector<ScaFES::DataField<TT, DIM>>&, const std::vector<ScaFES::DataField<TT, DIM>>&, const ScaFES::Ntuple<int, DIM>&, const int&) {}
    template <typename TT>
    void updateBorder2(std::vector<ScaFES::DataField<TT, DIM>>&, const std::vector<ScaFES::DataField<TT, DIM>>&, const ScaFES::Ntuple<int, DIM>&, const int&) {}
    const std::vector<ScaFES::DataField<CT, DIM>>& latest() const { return this->mVectUnknownDfsDomOld; }
};

template <typename CT, std::size_t DIM, int KIND>
class HeatFlux : public ScaFES::Problem<HeatFlux<CT, DIM, KIND>, CT, DIM> {
    using Base = ScaFES::Problem<HeatFlux<CT, DIM, KIND>, CT, DIM>;
public:
    using Base::Base;
    const double RHO = 1.0, C = 1.0, LAMBDA = 1.0, ALPHA = 1.0;
    bool onMin(const ScaFES::Ntuple<int, DIM>& n) const {
        for (std::size_t p = 0; p < DIM; ++p)
            if (n[p] == 0) return true;
        return false;
    }
    void evalInner(std::vector<ScaFES::DataField<CT, DIM>>& v, const ScaFES::Ntuple<int, DIM>& n, const int& t) {
        const double s = HeatLin<CT, DIM>::lin(this->coordinates(n));
        v[0](n) = s * (RHO * C);
        v[1](n) = 0.0;
        v[2](n) = s * (1.0 + this->time(t));
    }
    void evalBorder(std::vector<ScaFES::DataField<CT, DIM>>& v, const ScaFES::Ntuple<int, DIM>& n, const int& t) {
        const double s = HeatLin<CT, DIM>::lin(this->coordinates(n));
        const double tt = this->time(t);
        v[0](n) = s * (RHO * C);
        if (onMin(n)) v[1](n) = s * (1.0 + tt);
        else if (KIND == 0) v[1](n) = -1.0 * LAMBDA * (1.0 + tt);
        else v[1](n) = s * (ALPHA * (1.0 + tt)) + LAMBDA * (1.0 + tt);
        v[2](n) = s * (1.0 + tt);
    }
    template <typename TT>
    void initInner(std::vector<ScaFES::DataField<TT, DIM>>& v, const std::vector<TT>&, const ScaFES::Ntuple<int, DIM>& n, const int& t) {
        v[0](n) = HeatLin<CT, DIM>::lin(this->coordinates(n)) * (1.0 + this->time(t));
    }
    template <typename TT>
    void initBorder(std::vector<ScaFES::DataField<TT, DIM>>& v, const std::vector<TT>& o, const ScaFES::Ntuple<int, DIM>& n, const int& t) {
        initInner<TT>(v, o, n, t);
    }
    template <typename TT>
    void updateInner(std::vector<ScaFES::DataField<TT, DIM>>& vNew, const std::vector<ScaFES::DataField<TT, DIM>>& vOld,
                     const ScaFES::Ntuple<int, DIM>& n, const int&) {
        vNew[0](n) = vOld[0](n);
        for (std::size_t p = 0; p < DIM; ++p)
            vNew[0](n) += this->tau() * (LAMBDA / (RHO * C)) *
                          (vOld[0](this->connect(n, 2 * p)) + vOld[0](this->connect(n, 2 * p + 1)) - 2.0 * vOld[0](n)) /
                          (this->gridsize(p) * this->gridsize(p));
        vNew[0](n) += this->tau() * (1.0 / (RHO * C)) * this->knownDfOld(0, n);
    }
    template <typename TT>
    void updateBorder(std::vector<ScaFES::DataField<TT, DIM>>& vNew, const std::vector<ScaFES::DataField<TT, DIM>>& vOld,
                      const ScaFES::Ntuple<int, DIM>& n, const int&) {
        if (onMin(n)) {
            vNew[0](n) = this->knownDf(1, n);
            return;
        }
        vNew[0](n) = vOld[0](n);
        for (std::size_t p = 0; p < DIM; ++p) {
            const double h = this->gridsize(p);
            if (n[p] == this->nNodes(p) - 1) {
                // The missing outer neighbour is the mirrored inner one; the
                // flux condition enters through the border field.
                if (KIND == 0)
                    vNew[0](n) += this->tau() * (LAMBDA / (RHO * C)) *
                                  (vOld[0](this->connect(n, 2 * p)) + vOld[0](this->connect(n, 2 * p)) -
                                   ((2.0 * h / LAMBDA) * this->knownDfOld(1, n)) - 2.0 * vOld[0](n)) / (h * h);
                else
                    vNew[0](n) += this->tau() * (LAMBDA / (RHO * C)) *
                                  (vOld[0](this->connect(n, 2 * p)) + vOld[0](this->connect(n, 2 * p)) -
                                   ((2.0 * h / LAMBDA) * ALPHA * vOld[0](n)) +
                                   ((2.0 * h / LAMBDA) * this->knownDfOld(1, n)) - 2.0 * vOld[0](n)) / (h * h);
            } else {
                vNew[0](n) += this->tau() * (LAMBDA / (RHO * C)) *
                              (vOld[0](this->connect(n, 2 * p)) + vOld[0](this->connect(n, 2 * p + 1)) - 2.0 * vOld[0](n)) /
                              (h * h);
            }
        }
        vNew[0](n) += this->tau() * (1.0 / (RHO * C)) * this->knownDfOld(0, n);
    }
    template <typename TT>
    void updateInner2(std::vector<ScaFES::DataField<TT, DIM>>&, const std::vector<ScaFES::DataField<TT, DIM>>&, const ScaFES::Ntuple<int, DIM>&, const int&) {}
    template <typename TT>
    void updateBorder2(std::vector<ScaFES::DataField<TT, DIM>>&, const std::vector<ScaFES::DataField<TT, DIM>>&, const ScaFES::Ntuple<int, DIM>&, const int&) {}
    const std::vector<ScaFES::DataField<CT, DIM>>& latest() const { return this->mVectUnknownDfsDomOld; }
};

template <typename CT, std::size_t DIM>
class PennesRadiation : public ScaFES::Problem<PennesRadiation<CT, DIM>, CT, DIM> {
    using Base = ScaFES::Problem<PennesRadiation<CT, DIM>, CT, DIM>;
public:
    using Base::Base;
    const double RHO = 1.0, C = 1.0, LAMBDA = 1.0, RHO_B = 1.0, C_B = 1.0, W = 1.0, SIGMA = 1.0, EPS = 1.0;
    bool onMin(const ScaFES::Ntuple<int, DIM>& n) const {
        for (std::size_t p = 0; p < DIM; ++p)
            if (n[p] == 0) return true;
        return false;
    }
    double source(double s, double tt) const { return s * (RHO * C) + RHO_B * C_B * W * (s * (1.0 + tt)); }
    void evalInner(std::vector<ScaFES::DataField<CT, DIM>>& v, const ScaFES::Ntuple<int, DIM>& n, const int& t) {
        const double s = HeatLin<CT, DIM>::lin(this->coordinates(n));
        v[0](n) = source(s, this->time(t));
        v[1](n) = 0.0;
        v[2](n) = s * (1.0 + this->time(t));
    }
    void evalBorder(std::vector<ScaFES::DataField<CT, DIM>>& v, const ScaFES::Ntuple<int, DIM>& n, const int& t) {
        const double s = HeatLin<CT, DIM>::lin(this->coordinates(n));
        const double tt = this->time(t), y = s * (1.0 + tt);
        v[0](n) = source(s, tt);
        v[1](n) = onMin(n) ? y : ((y * y) * y) * y * (SIGMA * EPS) + LAMBDA * (1.0 + tt);
        v[2](n) = y;
    }
    template <typename TT>
    void initInner(std::vector<ScaFES::DataField<TT, DIM>>& v, const std::vector<TT>&, const ScaFES::Ntuple<int, DIM>& n, const int& t) {
        v[0](n) = HeatLin<CT, DIM>::lin(this->coordinates(n)) * (1.0 + this->time(t));
    }
    template <typename TT>
    void initBorder(std::vector<ScaFES::DataField<TT, DIM>>& v, const std::vector<TT>& o, const ScaFES::Ntuple<int, DIM>& n, const int& t) {
        initInner<TT>(v, o, n, t);
    }
    template <typename TT>
    void updateInner(std::vector<ScaFES::DataField<TT, DIM>>& vNew, const std::vector<ScaFES::DataField<TT, DIM>>& vOld,
                     const ScaFES::Ntuple<int, DIM>& n, const int&) {
        vNew[0](n) = vOld[0](n);
        for (std::size_t p = 0; p < DIM; ++p)
            vNew[0](n) += this->tau() * (LAMBDA / (RHO * C)) *
                          (vOld[0](this->connect(n, 2 * p)) + vOld[0](this->connect(n, 2 * p + 1)) - 2.0 * vOld[0](n)) /
                          (this->gridsize(p) * this->gridsize(p));
        vNew[0](n) -= this->tau() * ((RHO_B * C_B) / (RHO * C)) * W * vOld[0](n);
        vNew[0](n) += this->tau() * (1.0 / (RHO * C)) * this->knownDfOld(0, n);
    }
    template <typename TT>
    void updateBorder(std::vector<ScaFES::DataField<TT, DIM>>& vNew, const std::vector<ScaFES::DataField<TT, DIM>>& vOld,
                      const ScaFES::Ntuple<int, DIM>& n, const int&) {
        using std::pow;
        if (onMin(n)) {
            vNew[0](n) = this->knownDf(1, n);
            return;
        }
        vNew[0](n) = vOld[0](n);
        for (std::size_t p = 0; p < DIM; ++p) {
            const double h = this->gridsize(p);
            if (n[p] == this->nNodes(p) - 1) {
                // Mirrored inner neighbour; radiative loss eps sigma u^4 and
                // the border field enter as the flux.
                const double k = 2.0 * h / LAMBDA;
                vNew[0](n) += this->tau() * (LAMBDA / (RHO * C)) *
                              (2.0 * vOld[0](this->connect(n, 2 * p)) - k * (EPS * SIGMA) * pow(vOld[0](n), 4.0) +
                               k * this->knownDfOld(1, n) - 2.0 * vOld[0](n)) / (h * h);
            } else {
                vNew[0](n) += this->tau() * (LAMBDA / (RHO * C)) *
                              (vOld[0](this->connect(n, 2 * p)) + vOld[0](this->connect(n, 2 * p + 1)) - 2.0 * vOld[0](n)) /
                              (h * h);
            }
        }
        vNew[0](n) -= this->tau() * ((RHO_B * C_B) / (RHO * C)) * W * vOld[0](n);
        vNew[0](n) += this->tau() * (1.0 / (RHO * C)) * this->knownDfOld(0, n);
    }
    template <typename TT>
    void updateInner2(std::vector<ScaFES::DataField<TT, DIM>>&, const std::vector<ScaFES::DataField<TT, DIM>>&, const ScaFES::Ntuple<int, DIM>&, const int&) {}
    template <typename TT>
    void updateBorder2(std::vector<ScaFES::DataField<TT, DIM>>&, const std::vector<ScaFES::DataField<TT, DIM>>&, const ScaFES::Ntuple<int, DIM>&, const int&) {}
    const std::vector<ScaFES::DataField<CT, DIM>>& latest() const { return this->mVectUnknownDfsDomOld; }
};


// The tissue examples' update of one node: the axis brackets (a missing
// neighbour replaced by the inner one plus a flux term at a border face),
// then perfusion and heat source.  zmax(...) gives the z-max face's bracket.
template <class Prob, typename TT, std::size_t DIM, class ZMax>
void tissue_update(Prob& pb, std::vector<ScaFES::DataField<TT, DIM>>& vNew,
                   const std::vector<ScaFES::DataField<TT, DIM>>& vOld, const ScaFES::Ntuple<int, DIM>& n,
                   bool border, double rho, double c, double k, double rho_b, double c_b, double omega,
                   double t_b, double q, double q_bc, ZMax zmax) {
    const auto& U = vOld[0];
    vNew[0](n) = U(n);
    for (std::size_t p = 0; p < DIM; ++p) {
        const double h = pb.gridsize(p);
        const double cf = pb.tau() * (k / (rho * c));
        if (border && n.elem(p) == pb.nNodes(p) - 1) {
            if (p == DIM - 1) {
                vNew[0](n) += cf * zmax(U(pb.connect(n, 2 * p)), U(n), h, k, vNew[0](n)) / (h * h);
            } else {
                vNew[0](n) += cf * (U(pb.connect(n, 2 * p)) + U(pb.connect(n, 2 * p)) - ((2.0 * h / k) * (-1.0 * q_bc)) -
                                    2.0 * U(n)) / (h * h);
            }
        } else if (border && n.elem(p) == 0) {
            vNew[0](n) += cf * (U(pb.connect(n, 2 * p + 1)) + ((2.0 * h / k) * q_bc) + U(pb.connect(n, 2 * p + 1)) -
                                2.0 * U(n)) / (h * h);
        } else {
            vNew[0](n) += cf * (U(pb.connect(n, 2 * p)) + U(pb.connect(n, 2 * p + 1)) - 2.0 * U(n)) / (h * h);
        }
    }
    vNew[0](n) += pb.tau() * ((rho_b * c_b) / (rho * c)) * omega * (t_b - U(n));
    vNew[0](n) += pb.tau() * (1.0 / (rho * c)) * q;
}

template <typename CT, std::size_t DIM>
class TissueTumour : public ScaFES::Problem<TissueTumour<CT, DIM>, CT, DIM> {
    using Base = ScaFES::Problem<TissueTumour<CT, DIM>, CT, DIM>;
public:
    using Base::Base;
    // RHO C K Q_BRAIN Q_TUMOR RHO_B C_PB OMEGA_B_BRAIN OMEGA_B_TUMOR T_I H T_INF Q_BC DIAMETER DEPTH T_A
    double P[16] = {};
    double radius = 0.0;
    ScaFES::Ntuple<double, DIM> centre;
    void setParams(const std::vector<double>& v) {
        for (int i = 0; i < 16; ++i) P[i] = v.at(i);
        radius = P[13] / 2.0;
        for (std::size_t p = 0; p < DIM; ++p)
            centre[p] = p == DIM - 1 ? this->params().coordNodeLast()[p] - P[14] : this->params().coordNodeLast()[p] / 2.0;
    }
    void sphere(const ScaFES::Ntuple<int, DIM>& n, double& omega, double& q) const {
        const ScaFES::Ntuple<double, DIM> x = this->coordinates(n);
        double d = 0.0;
        for (std::size_t p = 0; p < DIM; ++p) d += (x[p] - centre[p]) * (x[p] - centre[p]);
        const bool in = d <= radius * radius;
        omega = in ? P[8] : P[7];
        q = in ? P[4] : P[3];
    }
    void evalInner(std::vector<ScaFES::DataField<CT, DIM>>&, const ScaFES::Ntuple<int, DIM>&, const int&) {}
    void evalBorder(std::vector<ScaFES::DataField<CT, DIM>>&, const ScaFES::Ntuple<int, DIM>&, const int&) {}
    template <typename TT>
    void initInner(std::vector<ScaFES::DataField<TT, DIM>>& v, const std::vector<TT>&, const ScaFES::Ntuple<int, DIM>& n,
                   const int&) {
        v[0](n) = P[9];
    }
    template <typename TT>
    void initBorder(std::vector<ScaFES::DataField<TT, DIM>>& v, const std::vector<TT>& o, const ScaFES::Ntuple<int, DIM>& n,
                    const int& t) {
        initInner<TT>(v, o, n, t);
    }
    template <typename TT>
    void update(std::vector<ScaFES::DataField<TT, DIM>>& vNew, const std::vector<ScaFES::DataField<TT, DIM>>& vOld,
                const ScaFES::Ntuple<int, DIM>& n, bool border) {
        double omega, q;
        sphere(n, omega, q);
        const double H = P[10], T_INF = P[11];
        auto cauchy = [&](const TT& a, const TT& u, double h, double k, const TT&) {
            return a + a - ((2.0 * h / k) * H * (u - T_INF)) - 2.0 * u;
        };
        tissue_update(*this, vNew, vOld, n, border, P[0], P[1], P[2], P[5], P[6], omega, P[15], q, P[12], cauchy);
    }
    template <typename TT>
    void updateInner(std::vector<ScaFES::DataField<TT, DIM>>& vNew, const std::vector<ScaFES::DataField<TT, DIM>>& vOld,
                     const ScaFES::Ntuple<int, DIM>& n, const int&) {
        update<TT>(vNew, vOld, n, false);
    }
    template <typename TT>
    void updateBorder(std::vector<ScaFES::DataField<TT, DIM>>& vNew, const std::vector<ScaFES::DataField<TT, DIM>>& vOld,
                      const ScaFES::Ntuple<int, DIM>& n, const int&) {
        update<TT>(vNew, vOld, n, true);
    }
    template <typename TT>
    void updateInner2(std::vector<ScaFES::DataField<TT, DIM>>&, const std::vector<ScaFES::DataField<TT, DIM>>&, const ScaFES::Ntuple<int, DIM>&, const int&) {}
    template <typename TT>
    void updateBorder2(std::vector<ScaFES::DataField<TT, DIM>>&, const std::vector<ScaFES::DataField<TT, DIM>>&, const ScaFES::Ntuple<int, DIM>&, const int&) {}
    const std::vector<ScaFES::DataField<CT, DIM>>& latest() const { return this->mVectUnknownDfsDomOld; }
};

template <typename CT, std::size_t DIM>
class TissueMri : public ScaFES::Problem<TissueMri<CT, DIM>, CT, DIM> {
    using Base = ScaFES::Problem<TissueMri<CT, DIM>, CT, DIM>;
public:
    using Base::Base;
    double H = 0.0, T_AMB = 0.0, Q_BC = 0.0, Q_SKULL = 0.0, EPSILON = 0.0;
    const double SIGMA = 5.670373e-8;
    void setParams(const std::vector<double>& v) {
        H = v.at(0); T_AMB = v.at(1); Q_BC = v.at(2); Q_SKULL = v.at(3); EPSILON = v.at(4);
    }
    // The nine known fields (rho, c, lambda, rho_blood, c_blood, omega,
    // T_blood, q, surface), n values each, x fastest.
    void setFields(const std::vector<double>& f) {
        const auto& g = this->globalGrid().discreteDomain();
        const long long nn = g.nNodesTotal();
        for (long long m = 0; m < nn; ++m) {
            const ScaFES::Ntuple<int, DIM> n = g.idxNodeScalar2TupleStyleFortran(m);
            for (int i = 0; i < 9; ++i) {
                this->mVectKnownDfsDomNew[i](n) = f.at((std::size_t)(i * nn + m));
                this->mVectKnownDfsDomOld[i](n) = f.at((std::size_t)(i * nn + m));
            }
        }
    }
    void evalInner(std::vector<ScaFES::DataField<CT, DIM>>&, const ScaFES::Ntuple<int, DIM>&, const int&) {}
    void evalBorder(std::vector<ScaFES::DataField<CT, DIM>>&, const ScaFES::Ntuple<int, DIM>&, const int&) {}
    template <typename TT>
    void initInner(std::vector<ScaFES::DataField<TT, DIM>>&, const std::vector<TT>&, const ScaFES::Ntuple<int, DIM>&, const int&) {}
    template <typename TT>
    void initBorder(std::vector<ScaFES::DataField<TT, DIM>>&, const std::vector<TT>&, const ScaFES::Ntuple<int, DIM>&, const int&) {}
    template <typename TT>
    void update(std::vector<ScaFES::DataField<TT, DIM>>& vNew, const std::vector<ScaFES::DataField<TT, DIM>>& vOld,
                const ScaFES::Ntuple<int, DIM>& n, bool border) {
        CT fld[9];
        for (int i = 0; i < 9; ++i) fld[i] = this->knownDf(i, n);
        const int open = (int)fld[8];
        auto skull = [&](const TT& a, const TT& u, double h, double k, const TT& partial) -> TT {
            if (open == 1) {
                const TT t_old = partial + 273.15;
                const TT t_old4 = t_old * t_old * t_old * t_old;
                const double t_amb = T_AMB + 273.15;
                const double t_amb4 = t_amb * t_amb * t_amb * t_amb;
                return a + a - ((2.0 * h / k) * H * (u - T_AMB)) - ((2.0 * h / k) * EPSILON * SIGMA * (t_old4 - t_amb4)) -
                       2.0 * u;
            }
            return a + a - ((2.0 * h / k) * (-1.0 * Q_SKULL)) - 2.0 * u;
        };
        tissue_update(*this, vNew, vOld, n, border, fld[0], fld[1], fld[2], fld[3], fld[4], fld[5], fld[6], fld[7],
                      Q_BC, skull);
    }
    template <typename TT>
    void updateInner(std::vector<ScaFES::DataField<TT, DIM>>& vNew, const std::vector<ScaFES::DataField<TT, DIM>>& vOld,
                     const ScaFES::Ntuple<int, DIM>& n, const int&) {
        update<TT>(vNew, vOld, n, false);
    }
    template <typename TT>
    void updateBorder(std::vector<ScaFES::DataField<TT, DIM>>& vNew, const std::vector<ScaFES::DataField<TT, DIM>>& vOld,
                      const ScaFES::Ntuple<int, DIM>& n, const int&) {
        update<TT>(vNew, vOld, n, true);
    }
    template <typename TT>
    void updateInner2(std::vector<ScaFES::DataField<TT, DIM>>&, const std::vector<ScaFES::DataField<TT, DIM>>&, const ScaFES::Ntuple<int, DIM>&, const int&) {}
    template <typename TT>
    void updateBorder2(std::vector<ScaFES::DataField<TT, DIM>>&, const std::vector<ScaFES::DataField<TT, DIM>>&, const ScaFES::Ntuple<int, DIM>&, const int&) {}
    const std::vector<ScaFES::DataField<CT, DIM>>& latest() const { return this->mVectUnknownDfsDomOld; }
};

// Yee cavity.  Node (i,j,k) holds Ex at (i+1/2, j, k), Hx at (i, j+1/2,
// k+1/2) and so on; an H component exists where its two staggered
// directions have a node beyond, an E component where its own direction
// has one and the two others are inner (tangential E is 0 on the walls
// and stays at its initial value there).  The initial fields come from
// setFields (six fields of n nodes, x fastest).
template <typename CT, std::size_t DIM>
class YeeCavity : public ScaFES::Problem<YeeCavity<CT, DIM>, CT, DIM> {
    using Base = ScaFES::Problem<YeeCavity<CT, DIM>, CT, DIM>;
    using Tup = ScaFES::Ntuple<int, DIM>;
    std::vector<double> mInit;
    bool mVary = false;
public:
    using Base::Base;
    void setFields(const std::vector<double>& f) { mInit = f; }
    // A coefficient that differs at the single inner node (3, 3, 3) (a
    // medium that is not uniform), which the multi-field device form cannot
    // express; the node lies on none of the lines the first check probes.
    void setVarying(bool v) { mVary = v; }
    void evalInner(std::vector<ScaFES::DataField<CT, DIM>>&, const Tup&, const int&) {}
    void evalBorder(std::vector<ScaFES::DataField<CT, DIM>>&, const Tup&, const int&) {}
    template <typename TT>
    void initInner(std::vector<ScaFES::DataField<TT, DIM>>& v, const std::vector<TT>&, const Tup& n, const int&) {
        const auto& g = this->globalGrid().discreteDomain();
        const long long nn = g.nNodesTotal(), m = g.idxNodeTuple2ScalarStyleFortran(n);
        for (int c = 0; c < 6; ++c) v[c](n) = mInit.empty() ? 0.0 : mInit.at((std::size_t)(c * nn + m));
    }
    template <typename TT>
    void initBorder(std::vector<ScaFES::DataField<TT, DIM>>& v, const std::vector<TT>& o, const Tup& n, const int& t) {
        initInner<TT>(v, o, n, t);
    }
    // Has node n a neighbour in direction +p / is it inner in direction p?
    bool up(const Tup& n, int p) { return n[p] < this->globalGrid().discreteDomain().idxNodeLast(p); }
    bool in(const Tup& n, int p) {
        const auto& g = this->globalGrid().discreteDomain();
        return n[p] > g.idxNodeFirst(p) && n[p] < g.idxNodeLast(p);
    }
    template <typename TT>
    void hStep(std::vector<ScaFES::DataField<TT, DIM>>& vNew, const std::vector<ScaFES::DataField<TT, DIM>>& vOld,
               const Tup& n) {
        const bool odd = mVary && n[0] == 3 && n[1] == 3 && n[2] == 3;
        const double ch = this->tau() / this->gridsize(0) * (odd ? 1.001 : 1.0);
        const Tup px = this->connect(n, 1), py = this->connect(n, 3), pz = this->connect(n, 5);
        if (up(n, 1) && up(n, 2))
            vNew[3](n) = vOld[3](n) - ch * ((vOld[2](py) - vOld[2](n)) - (vOld[1](pz) - vOld[1](n)));
        if (up(n, 0) && up(n, 2))
            vNew[4](n) = vOld[4](n) - ch * ((vOld[0](pz) - vOld[0](n)) - (vOld[2](px) - vOld[2](n)));
        if (up(n, 0) && up(n, 1))
            vNew[5](n) = vOld[5](n) - ch * ((vOld[1](px) - vOld[1](n)) - (vOld[0](py) - vOld[0](n)));
    }
    template <typename TT>
    void eStep(std::vector<ScaFES::DataField<TT, DIM>>& vNew, const std::vector<ScaFES::DataField<TT, DIM>>& vOld,
               const Tup& n) {
        const double ch = this->tau() / this->gridsize(0);
        const Tup mx = this->connect(n, 0), my = this->connect(n, 2), mz = this->connect(n, 4);
        if (up(n, 0) && in(n, 1) && in(n, 2))
            vNew[0](n) = vOld[0](n) + ch * ((vOld[5](n) - vOld[5](my)) - (vOld[4](n) - vOld[4](mz)));
        if (up(n, 1) && in(n, 0) && in(n, 2))
            vNew[1](n) = vOld[1](n) + ch * ((vOld[3](n) - vOld[3](mz)) - (vOld[5](n) - vOld[5](mx)));
        if (up(n, 2) && in(n, 0) && in(n, 1))
            vNew[2](n) = vOld[2](n) + ch * ((vOld[4](n) - vOld[4](mx)) - (vOld[3](n) - vOld[3](my)));
    }
    template <typename TT>
    void updateInner(std::vector<ScaFES::DataField<TT, DIM>>& vNew, const std::vector<ScaFES::DataField<TT, DIM>>& vOld,
                     const Tup& n, const int&) {
        hStep<TT>(vNew, vOld, n);
    }
    template <typename TT>
    void updateBorder(std::vector<ScaFES::DataField<TT, DIM>>& vNew, const std::vector<ScaFES::DataField<TT, DIM>>& vOld,
                      const Tup& n, const int&) {
        hStep<TT>(vNew, vOld, n);
    }
    template <typename TT>
    void updateInner2(std::vector<ScaFES::DataField<TT, DIM>>& vNew, const std::vector<ScaFES::DataField<TT, DIM>>& vOld,
                      const Tup& n, const int&) {
        eStep<TT>(vNew, vOld, n);
    }
    template <typename TT>
    void updateBorder2(std::vector<ScaFES::DataField<TT, DIM>>& vNew, const std::vector<ScaFES::DataField<TT, DIM>>& vOld,
                       const Tup& n, const int&) {
        eStep<TT>(vNew, vOld, n);
    }
    const std::vector<ScaFES::DataField<CT, DIM>>& latest() const { return this->mVectUnknownDfsDomOld; }
};

// LameFirstOrder -- the update of the reference's first-order Lame-Navier
// example (examples/LameNavierEqnFDMFirstOrder/LameNavierEqnFDMFirstOrder.hpp:
// 393-520), restated statement by statement in the example's operation
// order so that the recorded rules are the same doubles: unknown fields
// U1 U2 U3 V1 V2 V3 (indices 0..5), known fields F1..F3, G1..G3 (zero in
// the example), material constants of the example.  Its statements are
// kept as the example has them, including the ones that look unintended
// (the third component's Laplacian accumulates into the first
// displacement; the first velocity starts from twice its old value): the
// point is to run what the reference runs.
template <typename CT, std::size_t DIM>
class LameFirstOrder : public ScaFES::Problem<LameFirstOrder<CT, DIM>, CT, DIM> {
    using Base = ScaFES::Problem<LameFirstOrder<CT, DIM>, CT, DIM>;
    using Tup = ScaFES::Ntuple<int, DIM>;
public:
    using Base::Base;
    const double E = 1.0e6, NU = 0.4999;
    const double LAMBDA = NU * E / ((1.0 + NU) * (1.0 - 2.0 * NU));
    const double MU = E / (2.0 * (1.0 + NU));
    const double RHO = 1.0, FREQ = 1.0;
    const double OMEGA = 2.0 * M_PI * FREQ;
    void evalInner(std::vector<ScaFES::DataField<CT, DIM>>& v, const Tup& n, const int& t) {
        for (int i = 0; i < 8; ++i) v[i](n) = 0.0;
        v[8](n) = OMEGA * std::cos(OMEGA * this->time(t));
    }
    void evalBorder(std::vector<ScaFES::DataField<CT, DIM>>& v, const Tup& n, const int& t) { evalInner(v, n, t); }
    template <typename TT>
    void initInner(std::vector<ScaFES::DataField<TT, DIM>>& v, const std::vector<TT>&, const Tup& n, const int& t) {
        const double w = OMEGA * this->time(t);
        for (int i = 0; i < 6; ++i) v[i](n) = 0.0;
        v[2](n) = std::sin(w);
        v[5](n) = OMEGA * std::cos(w);
    }
    template <typename TT>
    void initBorder(std::vector<ScaFES::DataField<TT, DIM>>& v, const std::vector<TT>& o, const Tup& n, const int& t) {
        initInner<TT>(v, o, n, t);
    }
    // t -= MU tau (2 s(n) - s(n-p) - s(n+p)) / hh, summed over the axes p.
    template <typename TT>
    void lap(std::vector<ScaFES::DataField<TT, DIM>>& vNew, const std::vector<ScaFES::DataField<TT, DIM>>& vOld,
             const Tup& n, int t, int s, bool with_rho) {
        for (std::size_t p = 0; p < DIM; ++p) {
            const double hh = with_rho ? this->gridsize(p) * this->gridsize(p) * RHO
                                       : this->gridsize(p) * this->gridsize(p);
            vNew[t](n) -= MU * this->tau() *
                          (2.0 * vOld[s](n) - vOld[s](this->connect(n, 2 * p)) - vOld[s](this->connect(n, 2 * p + 1))) /
                          hh;
        }
    }
    // t -= (MU + LAMBDA) tau (s(a) - s(b) - s(n) + s(d)) / hh
    template <typename TT>
    void mix(std::vector<ScaFES::DataField<TT, DIM>>& vNew, const std::vector<ScaFES::DataField<TT, DIM>>& vOld,
             const Tup& n, int t, int s, const Tup& a, const Tup& b, const Tup& d, double hh) {
        vNew[t](n) -= (MU + LAMBDA) * this->tau() * (vOld[s](a) - vOld[s](b) - vOld[s](n) + vOld[s](d)) / hh;
    }
    template <typename TT>
    void updateInner(std::vector<ScaFES::DataField<TT, DIM>>& vNew, const std::vector<ScaFES::DataField<TT, DIM>>& vOld,
                     const Tup& n, const int&) {
        auto c = [&](const Tup& m, int dir) { return this->connect(m, dir); };
        const double h0 = this->gridsize(0), h1 = this->gridsize(1), h2 = this->gridsize(2);
        for (int a = 0; a < 3; ++a) vNew[a](n) = vOld[a](n) + this->tau() * vOld[3 + a](n);
        vNew[3](n) += vOld[3](n);
        lap<TT>(vNew, vOld, n, 0, 0, true);
        mix<TT>(vNew, vOld, n, 3, 0, c(n, 1), n, c(n, 0), h0 * h0);
        mix<TT>(vNew, vOld, n, 3, 0, c(n, 3), c(c(n, 3), 0), c(n, 0), h0 * h1);
        mix<TT>(vNew, vOld, n, 3, 0, c(n, 5), c(c(n, 5), 0), c(n, 0), h0 * h2);
        vNew[3](n) -= this->tau() * this->knownDf(0, n);
        vNew[4](n) = vOld[4](n);
        lap<TT>(vNew, vOld, n, 1, 1, false);
        mix<TT>(vNew, vOld, n, 4, 1, c(n, 3), n, c(n, 2), h1 * h1);
        mix<TT>(vNew, vOld, n, 4, 1, c(n, 1), c(c(n, 1), 2), c(n, 2), h1 * h0);
        mix<TT>(vNew, vOld, n, 4, 1, c(n, 5), c(c(n, 5), 2), c(n, 2), h1 * h2);
        vNew[4](n) -= this->tau() * this->knownDf(1, n);
        vNew[5](n) = vOld[5](n);
        lap<TT>(vNew, vOld, n, 0, 2, false);
        mix<TT>(vNew, vOld, n, 5, 2, c(n, 1), n, c(n, 4), h2 * h2);
        mix<TT>(vNew, vOld, n, 5, 2, c(n, 1), c(c(n, 1), 4), c(n, 4), h2 * h1);
        mix<TT>(vNew, vOld, n, 5, 2, c(n, 3), c(c(n, 3), 4), c(n, 4), h2 * h2);
        vNew[5](n) -= this->tau() * this->knownDf(2, n);
    }
    template <typename TT>
    void updateBorder(std::vector<ScaFES::DataField<TT, DIM>>& vNew, const std::vector<ScaFES::DataField<TT, DIM>>& vOld,
                      const Tup& n, const int&) {
        for (int a = 0; a < 3; ++a) vNew[a](n) = vOld[a](n) + this->tau() * vOld[3 + a](n);
        for (int a = 0; a < 3; ++a) vNew[3 + a](n) = this->knownDf(3 + a, n);
    }
    template <typename TT>
    void updateInner2(std::vector<ScaFES::DataField<TT, DIM>>&, const std::vector<ScaFES::DataField<TT, DIM>>&, const Tup&, const int&) {}
    template <typename TT>
    void updateBorder2(std::vector<ScaFES::DataField<TT, DIM>>&, const std::vector<ScaFES::DataField<TT, DIM>>&, const Tup&, const int&) {}
    const std::vector<ScaFES::DataField<CT, DIM>>& latest() const { return this->mVectUnknownDfsDomOld; }
};
