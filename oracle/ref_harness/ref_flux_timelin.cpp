// Reference driver run of a flux-border system test: the TimeLinSpaceLin
// problem of tests/system/HeatEqnFDM/{Neumann,Cauchy} or
// tests/system/PennesBioheatEqnFDM/{Neumann,Cauchy,Radiation} -- which one
// is chosen by the include path the Makefile gives (each directory defines
// its own TimeLinSpaceLin class on top of its Neumann.hpp / Cauchy.hpp /
// Radiation.hpp).  Same field
// set as the reference's main3D.cpp of those directories.
#include "harness.hpp"
#include "TimeLinSpaceLin.hpp"

struct Latest : public TimeLinSpaceLin<double, 3> {
    using TimeLinSpaceLin<double, 3>::TimeLinSpaceLin;
    const std::vector<ScaFES::DataField<double, 3>>& latest() const { return this->mVectUnknownDfsDomOld; }
};

int main(int argc, char** argv) {
    harness::Config c = harness::parse(argc, argv);
    ScaFES::Parameters p(argc, argv);
    harness::apply(p, c, 3);
    ScaFES::GridGlobal<3> gg(p);
    std::vector<std::string> names{"F", "G", "U"};
    std::vector<int> sw{0, 0, 1};
    std::vector<bool> known{true, true, false};
    std::vector<int> nl{0, 0, 0};
    std::vector<double> dv{0.0, 0.0, 0.0};
    std::vector<ScaFES::WriteHowOften> wr(3, ScaFES::WriteHowOften::NEVER);
    std::vector<bool> ce{false, false, false};
    Latest ppp(p, gg, false, names, sw, known, nl, dv, wr, ce, std::vector<double>());
    ppp.iterateOverTime();
    std::vector<double> out;
    harness::collect(ppp.latest()[0], c, out);
    harness::write_raw(c.out, out);
    return 0;
}
