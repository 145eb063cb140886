// Reference driver run: tests/system/HeatEqnFdmStencilWidthVar (three fields
// of stencil width 0, 1, 2; exact solution i+j+k+2n).  Dumps the three final
// fields back to back.
#include "harness.hpp"
#include "HeatEqnFdmStencilWidthVar.hpp"

struct Latest : public HeatEqnFdmStencilWidthVar<double, 3> {
    using HeatEqnFdmStencilWidthVar<double, 3>::HeatEqnFdmStencilWidthVar;
    const std::vector<ScaFES::DataField<double, 3>>& latest() const { return this->mVectUnknownDfsDomOld; }
};

int main(int argc, char** argv) {
    harness::Config c = harness::parse(argc, argv);
    ScaFES::Parameters p(argc, argv);
    harness::apply(p, c, 3);
    ScaFES::GridGlobal<3> gg(p);
    // Field set of tests/system/HeatEqnFdmStencilWidthVar/main3D.cpp.
    std::vector<std::string> names{"A", "B", "C"};
    std::vector<int> sw{0, 1, 2};
    std::vector<bool> known(3, false);
    std::vector<int> nl(3, 0);
    std::vector<double> dv(3, 0.0);
    std::vector<ScaFES::WriteHowOften> wr(3, ScaFES::WriteHowOften::NEVER);
    std::vector<bool> ce(3, true);  // as main3D.cpp (the known copies are allocated only then)
    Latest ppp(p, gg, false, names, sw, known, nl, dv, wr, ce, std::vector<double>());
    ppp.iterateOverTime();
    std::vector<double> out;
    for (int f = 0; f < 3; ++f) harness::collect(ppp.latest()[f], c, out);
    harness::write_raw(c.out, out);
    return 0;
}
