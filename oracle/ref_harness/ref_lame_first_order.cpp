// Reference driver run of the reference's first-order Lame-Navier example,
// compiled from the UNMODIFIED examples/LameNavierEqnFDMFirstOrder/
// LameNavierEqnFDMFirstOrder.hpp: six unknown fields (displacements U1..U3
// and velocities V1..V3) coupled through updateInner/updateBorder, six
// known fields (forces F1..F3 and border velocities G1..G3, zero), the
// field set of the example's main.cpp.  The run is the reference's own
// iterateOverTime(); the six unknown fields at the end are written one
// after the other.  (The example's author notes that the scheme is not a
// usable Lame-Navier solver; it serves here as the reference's own
// multi-unknown class.)
#include "harness.hpp"

#include "LameNavierEqnFDMFirstOrder.hpp"

struct LameFirstOrderLatest : public LameNavierEqnFDMFirstOrder<double, 3> {
    using LameNavierEqnFDMFirstOrder<double, 3>::LameNavierEqnFDMFirstOrder;
    const std::vector<ScaFES::DataField<double, 3>>& latest() const { return this->mVectUnknownDfsDomOld; }
};

int main(int argc, char** argv) {
    harness::Config cfg = harness::parse(argc, argv);
    ScaFES::Parameters p(argc, argv);
    harness::apply(p, cfg, 3);
    ScaFES::GridGlobal<3> gg(p);
    std::vector<std::string> names{"F1", "F2", "F3", "G1", "G2", "G3", "U1", "U2", "U3", "V1", "V2", "V3"};
    std::vector<int> sw{0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 1, 1};
    std::vector<bool> known{true, true, true, true, true, true, false, false, false, false, false, false};
    std::vector<int> nl(12, 0);
    std::vector<double> dv(12, 0.0);
    std::vector<ScaFES::WriteHowOften> wr(12, ScaFES::WriteHowOften::NEVER);
    std::vector<bool> ce(12, false);
    LameFirstOrderLatest ppp(p, gg, false, names, sw, known, nl, dv, wr, ce, std::vector<double>());
    ppp.iterateOverTime();
    std::vector<double> out;
    for (const auto& df : ppp.latest()) harness::collect(df, cfg, out);
    harness::write_raw(cfg.out, out);
    return 0;
}
