// Reference driver run: heat equation (tests/system/HeatEqnFDM/HeatEqnFDM.hpp)
// with the reference's Dirichlet border class (tests/system/HeatEqnFDM/
// Dirichlet/Dirichlet.hpp), F = 0, G = 0 and the initial iterate read from a
// file (e.g. the sine mode of the heat workloads, optionally with noise).
#include "harness.hpp"
#include "Dirichlet.hpp"

static std::vector<double> g_u0;
static harness::Config g_cfg;

template <typename CT, std::size_t DIM>
class HeatFromArray : public Dirichlet<CT, DIM, HeatFromArray<CT, DIM>> {
public:
    using Base = Dirichlet<CT, DIM, HeatFromArray<CT, DIM>>;
    template <class... A>
    HeatFromArray(A&&... a) : Base(std::forward<A>(a)...) {}
    void evalInner(std::vector<ScaFES::DataField<CT, DIM>>& v, ScaFES::Ntuple<int, DIM> const& n, int const&) {
        v[0](n) = 0.0;
        v[1](n) = 0.0;
    }
    void evalBorder(std::vector<ScaFES::DataField<CT, DIM>>& v, ScaFES::Ntuple<int, DIM> const& n, int const& t) {
        evalInner(v, n, t);
    }
    template <typename TT>
    void initInner(std::vector<ScaFES::DataField<TT, DIM>>& v, std::vector<TT> const&,
                   ScaFES::Ntuple<int, DIM> const& n, int const&) {
        const size_t m = n[0] + (size_t)g_cfg.n[0] * (n[1] + (size_t)g_cfg.n[1] * n[2]);
        v[0](n) = g_u0[m];
    }
    template <typename TT>
    void initBorder(std::vector<ScaFES::DataField<TT, DIM>>& v, std::vector<TT> const& o,
                    ScaFES::Ntuple<int, DIM> const& n, int const& t) {
        this->template initInner<TT>(v, o, n, t);
    }
    const std::vector<ScaFES::DataField<CT, DIM>>& latest() const { return this->mVectUnknownDfsDomOld; }
};

int main(int argc, char** argv) {
    g_cfg = harness::parse(argc, argv);
    ScaFES::Parameters p(argc, argv);
    harness::apply(p, g_cfg, 3);
    ScaFES::GridGlobal<3> gg(p);
    g_u0 = harness::read_raw(g_cfg.in, (size_t)g_cfg.n[0] * g_cfg.n[1] * g_cfg.n[2]);
    std::vector<std::string> names{"F", "G", "U"};
    std::vector<int> sw{0, 0, 1};
    std::vector<bool> known{true, true, false};
    std::vector<int> nl{0, 0, 0};
    std::vector<double> dv{0.0, 0.0, 0.0};
    std::vector<ScaFES::WriteHowOften> wr(3, ScaFES::WriteHowOften::NEVER);
    std::vector<bool> ce{false, false, false};
    HeatFromArray<double, 3> ppp(p, gg, false, names, sw, known, nl, dv, wr, ce, std::vector<double>());
    ppp.iterateOverTime();
    std::vector<double> out;
    harness::collect(ppp.latest()[0], g_cfg, out);
    harness::write_raw(g_cfg.out, out);
    return 0;
}
