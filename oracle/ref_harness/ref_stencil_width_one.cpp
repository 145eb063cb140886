// Reference driver run: tests/system/HeatEqnFdmStencilWidthOne (exact
// solution 2^n (i+j+k)).
#include "harness.hpp"
#include "HeatEqnFdmStencilWidthOne.hpp"

struct Latest : public HeatEqnFdmStencilWidthOne<double, 3> {
    using HeatEqnFdmStencilWidthOne<double, 3>::HeatEqnFdmStencilWidthOne;
    const std::vector<ScaFES::DataField<double, 3>>& latest() const { return this->mVectUnknownDfsDomOld; }
};

int main(int argc, char** argv) {
    harness::Config c = harness::parse(argc, argv);
    ScaFES::Parameters p(argc, argv);
    harness::apply(p, c, 3);
    ScaFES::GridGlobal<3> gg(p);
    // Field set of tests/system/HeatEqnFdmStencilWidthOne/main3D.cpp.
    std::vector<std::string> names{"A"};
    std::vector<int> sw{1};
    std::vector<bool> known{false};
    std::vector<int> nl{0};
    std::vector<double> dv{0.0};
    std::vector<ScaFES::WriteHowOften> wr(1, ScaFES::WriteHowOften::NEVER);
    std::vector<bool> ce{true};  // as main3D.cpp (the known copy of the field is allocated only then)
    Latest ppp(p, gg, false, names, sw, known, nl, dv, wr, ce, std::vector<double>());
    ppp.iterateOverTime();
    std::vector<double> out;
    harness::collect(ppp.latest()[0], c, out);
    harness::write_raw(c.out, out);
    return 0;
}
