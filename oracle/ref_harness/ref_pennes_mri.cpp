// Reference driver run: variable-coefficient Pennes bioheat update in the
// form of examples/MRIDataPBHEqnFDM/MRIDataPBHEqnFDM.hpp:143-169 (that class
// itself needs Boost.PropertyTree, so its updateInner is written out here in
// the same operation order, with the coefficients as scalars), Dirichlet
// border from a known field, driven by the reference's Problem.
// in.bin holds u0, q and g back to back; argv[16..22] are
// rho c k rho_blood c_blood omega T_blood.
#include "harness.hpp"

static std::vector<double> g_in;
static harness::Config g_cfg;
static double g_rho, g_c, g_k, g_rho_b, g_c_b, g_omega, g_t_blood;

static size_t lin(const ScaFES::Ntuple<int, 3>& n) {
    return n[0] + (size_t)g_cfg.n[0] * (n[1] + (size_t)g_cfg.n[1] * n[2]);
}

template <typename CT, std::size_t DIM>
class PennesMri : public ScaFES::Problem<PennesMri<CT, DIM>, CT, DIM> {
public:
    using Base = ScaFES::Problem<PennesMri<CT, DIM>, CT, DIM>;
    template <class... A>
    PennesMri(A&&... a) : Base(std::forward<A>(a)...) {}
    size_t nn() const { return (size_t)g_cfg.n[0] * g_cfg.n[1] * g_cfg.n[2]; }
    void evalInner(std::vector<ScaFES::DataField<CT, DIM>>& v, ScaFES::Ntuple<int, DIM> const& n, int const&) {
        v[0](n) = g_in[nn() + lin(n)];
        v[1](n) = g_in[2 * nn() + lin(n)];
    }
    void evalBorder(std::vector<ScaFES::DataField<CT, DIM>>& v, ScaFES::Ntuple<int, DIM> const& n, int const& t) {
        evalInner(v, n, t);
    }
    template <typename TT>
    void initInner(std::vector<ScaFES::DataField<TT, DIM>>& v, std::vector<TT> const&,
                   ScaFES::Ntuple<int, DIM> const& n, int const&) {
        v[0](n) = g_in[lin(n)];
    }
    template <typename TT>
    void initBorder(std::vector<ScaFES::DataField<TT, DIM>>& v, std::vector<TT> const& o,
                    ScaFES::Ntuple<int, DIM> const& n, int const& t) {
        this->template initInner<TT>(v, o, n, t);
    }
    template <typename TT>
    void updateInner(std::vector<ScaFES::DataField<TT, DIM>>& vNew,
                     std::vector<ScaFES::DataField<TT, DIM>> const& vOld,
                     ScaFES::Ntuple<int, DIM> const& idxNode, int const&) {
        CT rho = g_rho, c = g_c, k = g_k, rho_blood = g_rho_b, c_blood = g_c_b, omega = g_omega;
        CT T_blood = g_t_blood;
        CT q = this->knownDf(0, idxNode);
        vNew[0](idxNode) = vOld[0](idxNode);
        for (std::size_t pp = 0; pp < DIM; ++pp) {
            vNew[0](idxNode) += this->tau() * (k / (rho * c)) *
                                (vOld[0](this->connect(idxNode, 2 * pp)) +
                                 vOld[0](this->connect(idxNode, 2 * pp + 1)) - 2.0 * vOld[0](idxNode)) /
                                (this->gridsize(pp) * this->gridsize(pp));
        }
        vNew[0](idxNode) += this->tau() * ((rho_blood * c_blood) / (rho * c)) * omega * (T_blood - vOld[0](idxNode));
        vNew[0](idxNode) += this->tau() * (1.0 / (rho * c)) * q;
    }
    template <typename TT>
    void updateBorder(std::vector<ScaFES::DataField<TT, DIM>>& vNew, std::vector<ScaFES::DataField<TT, DIM>> const&,
                      ScaFES::Ntuple<int, DIM> const& idxNode, int const&) {
        vNew[0](idxNode) = this->knownDf(1, idxNode);
    }
    template <typename TT>
    void updateInner2(std::vector<ScaFES::DataField<TT, DIM>>&, std::vector<ScaFES::DataField<TT, DIM>> const&,
                      ScaFES::Ntuple<int, DIM> const&, int const&) {}
    template <typename TT>
    void updateBorder2(std::vector<ScaFES::DataField<TT, DIM>>&, std::vector<ScaFES::DataField<TT, DIM>> const&,
                       ScaFES::Ntuple<int, DIM> const&, int const&) {}
    const std::vector<ScaFES::DataField<CT, DIM>>& latest() const { return this->mVectUnknownDfsDomOld; }
};

int main(int argc, char** argv) {
    g_cfg = harness::parse(argc, argv);
    if (argc < 23) {
        std::fprintf(stderr, "ref_pennes_mri: need rho c k rho_b c_b omega T_blood after in.bin\n");
        return 2;
    }
    g_rho = std::atof(argv[16]); g_c = std::atof(argv[17]); g_k = std::atof(argv[18]);
    g_rho_b = std::atof(argv[19]); g_c_b = std::atof(argv[20]); g_omega = std::atof(argv[21]);
    g_t_blood = std::atof(argv[22]);
    ScaFES::Parameters p(argc, argv);
    harness::apply(p, g_cfg, 3);
    ScaFES::GridGlobal<3> gg(p);
    g_in = harness::read_raw(g_cfg.in, 3 * (size_t)g_cfg.n[0] * g_cfg.n[1] * g_cfg.n[2]);
    std::vector<std::string> names{"Q", "G", "T"};
    std::vector<int> sw{0, 0, 1};
    std::vector<bool> known{true, true, false};
    std::vector<int> nl{0, 0, 0};
    std::vector<double> dv{0.0, 0.0, 0.0};
    std::vector<ScaFES::WriteHowOften> wr(3, ScaFES::WriteHowOften::NEVER);
    std::vector<bool> ce{false, false, false};
    PennesMri<double, 3> ppp(p, gg, false, names, sw, known, nl, dv, wr, ce, std::vector<double>());
    ppp.iterateOverTime();
    std::vector<double> out;
    harness::collect(ppp.latest()[0], g_cfg, out);
    harness::write_raw(g_cfg.out, out);
    return 0;
}
