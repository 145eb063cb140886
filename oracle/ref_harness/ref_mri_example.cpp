// Reference driver run of the reference's MRI-data bioheat example,
// compiled from the UNMODIFIED examples/MRIDataPBHEqnFDM/MRIDataPBHEqnFDM.hpp:
// Pennes bioheat whose coefficients rho, c, lambda, rho_blood, c_blood,
// omega, T_blood, q are known fields over the nodes, with the example's
// Neumann borders and, at the z-max face, Neumann under a closed skull or
// convection + radiation where the "surface" field is 1.  The example reads
// its fields from MRI files (its evalInner/evalBorder/initInner are empty);
// this program writes them into the problem's known data fields before
// iterateOverTime, where they stay.  The initial temperature is the
// unknown field's default value (the reference resets the unknown field to
// it before the empty initInner runs).
// in.bin holds the nine known fields (rho, c, lambda, rho_blood, c_blood,
// omega, T_blood, q, surface) back to back; argv[16..20] are the example's
// Parameters H, T_INF, Q_BC, Q_SKULL, EPSILON and argv[21] the initial
// temperature.
#include "harness.hpp"

#include "MRIDataPBHEqnFDM.hpp"

struct MriLatest : public MRIDataPBHEqnFDM<double, 3> {
    using MRIDataPBHEqnFDM<double, 3>::MRIDataPBHEqnFDM;
    const std::vector<ScaFES::DataField<double, 3>>& latest() const { return this->mVectUnknownDfsDomOld; }
    // Known field f (0..8) from in.bin.
    void fill(const std::vector<double>& in, const harness::Config& c) {
        const size_t nn = (size_t)c.n[0] * c.n[1] * c.n[2];
        for (int k = 0; k < c.n[2]; ++k)
            for (int j = 0; j < c.n[1]; ++j)
                for (int i = 0; i < c.n[0]; ++i) {
                    ScaFES::Ntuple<int, 3> n;
                    n[0] = i;
                    n[1] = j;
                    n[2] = k;
                    const size_t m = i + (size_t)c.n[0] * (j + (size_t)c.n[1] * k);
                    for (int f = 0; f < 9; ++f) {
                        this->mVectKnownDfsDomNew[f](n) = in[f * nn + m];
                        this->mVectKnownDfsDomOld[f](n) = in[f * nn + m];
                    }
                }
    }
};

int main(int argc, char** argv) {
    static const char* NAMES[] = {"H", "T_INF", "Q_BC", "Q_SKULL", "EPSILON"};
    harness::Config cfg = harness::parse(argc, argv);
    if (argc < 22) {
        std::fprintf(stderr, "ref_mri_example: need H T_INF Q_BC Q_SKULL EPSILON T_INIT after in.bin\n");
        return 2;
    }
    boost::property_tree::ptree pt;
    for (int i = 0; i < 5; ++i) pt.put(std::string("Parameters.") + NAMES[i], std::atof(argv[16 + i]));
    ScaFES::Parameters p(argc, argv);
    harness::apply(p, cfg, 3);
    ScaFES::GridGlobal<3> gg(p);
    std::vector<std::string> names{"rho", "c", "lambda", "rho_blood", "c_blood", "omega", "T_blood", "q",
                                   "surface", "T"};
    std::vector<int> sw(10, 0);
    sw[9] = 1;
    std::vector<bool> known(10, true);
    known[9] = false;
    std::vector<int> nl(10, 0);
    std::vector<double> dv(10, 0.0);
    dv[9] = std::atof(argv[21]);
    std::vector<ScaFES::WriteHowOften> wr(10, ScaFES::WriteHowOften::NEVER);
    std::vector<bool> ce(10, false);
    std::vector<bool> conv(10, false);
    MriLatest ppp(p, gg, false, names, sw, known, pt, nl, dv, wr, ce, std::vector<double>(), conv);
    const size_t nn = (size_t)cfg.n[0] * cfg.n[1] * cfg.n[2];
    ppp.fill(harness::read_raw(cfg.in, 9 * nn), cfg);
    ppp.iterateOverTime();
    std::vector<double> out;
    harness::collect(ppp.latest()[0], cfg, out);
    harness::write_raw(cfg.out, out);
    return 0;
}
