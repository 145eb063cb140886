// Forward-mode derivative of the reference's own heat update
// (tests/system/HeatEqnFDM/HeatEqnFDM.hpp:205-218 updateInner<TT> with the
// Dirichlet updateBorder<TT> of tests/system/HeatEqnFDM/Dirichlet/
// Dirichlet.hpp:125-131), obtained the way the reference gets gradients: by
// instantiating its templated callbacks with a differentiable scalar (the
// hook ADOL-C's adouble uses, src/ScaFES_Problem.hpp:5646-5652; ADOL-C
// itself is not available here).  The scalar below is a dual number
// (value, derivative along one direction).  The time loop follows
// iterateOverTime's update phase (src/ScaFES_Problem.hpp:2596-2603,
// 5078-5082, 5419-5466): every node of the new iterate starts as a copy of
// the old one, border nodes run updateBorder, inner nodes updateInner,
// then old and new are swapped.
// in.bin holds u0 and the directions d_1..d_m (m = argv[16]); out.bin
// receives u_T and du_T along each direction.
#include "harness.hpp"
#include "Dirichlet.hpp"

struct Dual {
    double v = 0.0, d = 0.0;
    Dual() = default;
    Dual(double x) : v(x) {}
    Dual(int x) : v(x) {}
    Dual(double x, double y) : v(x), d(y) {}
    Dual& operator+=(const Dual& o) { v += o.v; d += o.d; return *this; }
    Dual& operator-=(const Dual& o) { v -= o.v; d -= o.d; return *this; }
    Dual& operator*=(const Dual& o) { d = d * o.v + v * o.d; v *= o.v; return *this; }
    Dual& operator/=(const Dual& o) {
        const double q = v / o.v;
        d = (d - q * o.d) / o.v;  // (d - (v/w) dw) / w: exact d / w for a constant divisor
        v = q;
        return *this;
    }
};
inline Dual operator+(Dual a, const Dual& b) { return a += b; }
inline Dual operator-(Dual a, const Dual& b) { return a -= b; }
inline Dual operator*(Dual a, const Dual& b) { return a *= b; }
inline Dual operator/(Dual a, const Dual& b) { return a /= b; }
inline Dual operator-(const Dual& a) { return Dual(-a.v, -a.d); }
inline bool operator<(const Dual& a, const Dual& b) { return a.v < b.v; }
inline bool operator>(const Dual& a, const Dual& b) { return a.v > b.v; }

static std::vector<double> g_in;
static harness::Config g_cfg;

template <typename CT, std::size_t DIM>
class HeatTangent : public Dirichlet<CT, DIM, HeatTangent<CT, DIM>> {
public:
    using Base = Dirichlet<CT, DIM, HeatTangent<CT, DIM>>;
    template <class... A>
    HeatTangent(A&&... a) : Base(std::forward<A>(a)...) {}
    void evalInner(std::vector<ScaFES::DataField<CT, DIM>>& v, ScaFES::Ntuple<int, DIM> const& n, int const&) {
        v[0](n) = 0.0;
        v[1](n) = 0.0;
    }
    void evalBorder(std::vector<ScaFES::DataField<CT, DIM>>& v, ScaFES::Ntuple<int, DIM> const& n, int const& t) {
        evalInner(v, n, t);
    }
    template <typename TT>
    void initInner(std::vector<ScaFES::DataField<TT, DIM>>&, std::vector<TT> const&, ScaFES::Ntuple<int, DIM> const&,
                   int const&) {}
    template <typename TT>
    void initBorder(std::vector<ScaFES::DataField<TT, DIM>>&, std::vector<TT> const&, ScaFES::Ntuple<int, DIM> const&,
                    int const&) {}

    // nsteps update phases on dual-number copies of the unknown field,
    // seeded with (u0, direction); returns u_T and du_T in Fortran order.
    void tangent(const double* u0, const double* dir, int nsteps, std::vector<double>& uT, std::vector<double>& duT) {
        const ScaFES::DataField<CT, DIM>& proto = this->mVectUnknownDfsDomNew[0];
        const ScaFES::Grid<DIM>& memAll = proto.memAll();
        const std::size_t nmem = memAll.nNodes().size() + 1;
        std::vector<Dual> a(nmem), b(nmem);
        std::vector<ScaFES::DataField<Dual, DIM>> vOld, vNew;
        vOld.emplace_back("Uold", &this->mParams, this->globalGrid(), memAll, proto.stencilWidth(), a.data());
        vNew.emplace_back("Unew", &this->mParams, this->globalGrid(), memAll, proto.stencilWidth(), b.data());
        const int nx = g_cfg.n[0], ny = g_cfg.n[1], nz = g_cfg.n[2];
        auto each = [&](auto fn) {
            for (int k = 0; k < nz; ++k)
                for (int j = 0; j < ny; ++j)
                    for (int i = 0; i < nx; ++i) {
                        ScaFES::Ntuple<int, DIM> n;
                        n[0] = i; n[1] = j; n[2] = k;
                        fn(n, (std::size_t)i + (std::size_t)nx * (j + (std::size_t)ny * k), i, j, k);
                    }
        };
        each([&](const ScaFES::Ntuple<int, DIM>& n, std::size_t m, int, int, int) { vOld[0](n) = Dual(u0[m], dir[m]); });
        const int L = this->mParams.nLayersAtBorder();
        for (int t = 1; t <= nsteps; ++t) {
            each([&](const ScaFES::Ntuple<int, DIM>& n, std::size_t, int, int, int) { vNew[0](n) = vOld[0](n); });
            each([&](const ScaFES::Ntuple<int, DIM>& n, std::size_t, int i, int j, int k) {
                const bool border = i < L || j < L || k < L || i > nx - 1 - L || j > ny - 1 - L || k > nz - 1 - L;
                if (border) this->template updateBorder<Dual>(vNew, vOld, n, t);
                else this->template updateInner<Dual>(vNew, vOld, n, t);
            });
            std::swap(vOld, vNew);
        }
        uT.resize((std::size_t)nx * ny * nz);
        duT.resize(uT.size());
        each([&](const ScaFES::Ntuple<int, DIM>& n, std::size_t m, int, int, int) {
            uT[m] = vOld[0](n).v;
            duT[m] = vOld[0](n).d;
        });
    }
};

int main(int argc, char** argv) {
    g_cfg = harness::parse(argc, argv);
    if (argc < 17) {
        std::fprintf(stderr, "ref_heat_tangent: need the number of directions after in.bin\n");
        return 2;
    }
    const int ndir = std::atoi(argv[16]);
    ScaFES::Parameters p(argc, argv);
    harness::apply(p, g_cfg, 3);
    ScaFES::GridGlobal<3> gg(p);
    const size_t nn = (size_t)g_cfg.n[0] * g_cfg.n[1] * g_cfg.n[2];
    g_in = harness::read_raw(g_cfg.in, (1 + (size_t)ndir) * nn);
    std::vector<std::string> names{"F", "G", "U"};
    std::vector<int> sw{0, 0, 1};
    std::vector<bool> known{true, true, false};
    std::vector<int> nl{0, 0, 0};
    std::vector<double> dv{0.0, 0.0, 0.0};
    std::vector<ScaFES::WriteHowOften> wr(3, ScaFES::WriteHowOften::NEVER);
    std::vector<bool> ce{false, false, false};
    HeatTangent<double, 3> ppp(p, gg, false, names, sw, known, nl, dv, wr, ce, std::vector<double>());
    std::vector<double> out, uT, duT;
    for (int d = 0; d < ndir; ++d) {
        ppp.tangent(g_in.data(), g_in.data() + (1 + (size_t)d) * nn, g_cfg.nsteps, uT, duT);
        if (d == 0) out.insert(out.end(), uT.begin(), uT.end());
        out.insert(out.end(), duT.begin(), duT.end());
    }
    harness::write_raw(g_cfg.out, out);
    return 0;
}
