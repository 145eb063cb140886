// Compiles one of the reference's own system-test problem classes,
// unchanged, against the drop-in headers and prints the device form its
// update maps to (test infrastructure; built only where the reference
// checkout is present).  PROBLEM selects the class and the field set of
// the matching reference main3D.cpp:
//   1 HeatEqnFDM/Dirichlet/TimeLinSpaceLin        2 PennesBioheatEqnFDM/Dirichlet/TimeLinSpaceLin
//   3 HeatEqnFdmStencilWidthOne                   4 HeatEqnFDM/Neumann/TimeLinSpaceLin
//   5 PropagationFromLeftLowerCorner              6 HeatEqnFDM/Cauchy/TimeLinSpaceLin
//   7 PennesBioheatEqnFDM/Neumann/TimeLinSpaceLin 8 PennesBioheatEqnFDM/Radiation/TimeLinSpaceLin
//   9 examples/TumorHeatEqnFDM                   10 examples/MRIDataPBHEqnFDM
//  11 examples/LameNavierEqnFDMFirstOrder (six unknown fields)
// (the examples need Boost.PropertyTree for their constants: the stand-in
// of oracle/ref_harness/stub goes on the include path).  Options:
//   --dump=PATH       also write the device form to PATH (dumpDeviceForm)
//   --params=a,b,...  the example's constants (tumour: the 16 of its
//                     Parameters.ini in TumorHeatEqnFDM order; MRI: H T_INF
//                     Q_BC Q_SKULL EPSILON T_INIT)
//   --fields=PATH     MRI: its nine known fields, raw FP64
//   --run=PATH        run iterateOverTime() on the GPU and write every
//                     unknown field of the final iterate to PATH
#include <cstdio>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "ScaFES.hpp"
#if PROBLEM == 9
#include "TumorHeatEqnFDM.hpp"
#elif PROBLEM == 10
#include "MRIDataPBHEqnFDM.hpp"
// Writes the known fields into the example's data fields (the example reads
// them from MRI files in its own main).
struct MriFilled : public MRIDataPBHEqnFDM<double, 3> {
    using MRIDataPBHEqnFDM<double, 3>::MRIDataPBHEqnFDM;
    void setFields(const std::vector<double>& f) {
        const auto& g = this->globalGrid().discreteDomain();
        const long long nn = g.nNodesTotal();
        for (long long m = 0; m < nn; ++m) {
            const ScaFES::Ntuple<int, 3> n = g.idxNodeScalar2TupleStyleFortran(m);
            for (int i = 0; i < 9; ++i) {
                this->mVectKnownDfsDomNew[i](n) = f.at((std::size_t)(i * nn + m));
                this->mVectKnownDfsDomOld[i](n) = f.at((std::size_t)(i * nn + m));
            }
        }
    }
};
#endif
#if PROBLEM == 11
#include "LameNavierEqnFDMFirstOrder.hpp"
#endif
// The final iterate (the "old" set after the last swap) of a problem class.
template <class P>
struct Latest : public P {
    using P::P;
    const std::vector<ScaFES::DataField<double, 3>>& latest() const { return this->mVectUnknownDfsDomOld; }
};
#if PROBLEM == 1 || PROBLEM == 2 || PROBLEM == 4 || PROBLEM == 6 || PROBLEM == 7 || PROBLEM == 8
#include "TimeLinSpaceLin.hpp"
#define CLASS TimeLinSpaceLin
#elif PROBLEM == 3
#include "HeatEqnFdmStencilWidthOne.hpp"
#define CLASS HeatEqnFdmStencilWidthOne
#elif PROBLEM == 5
#include "PropagationFromLeftLowerCorner.hpp"
#define CLASS PropagationFromLeftLowerCorner
#endif

static std::vector<double> read_doubles(const std::string& path) {
    std::vector<double> v;
    FILE* f = std::fopen(path.c_str(), "rb");
    double x;
    while (f && std::fread(&x, sizeof(double), 1, f) == 1) v.push_back(x);
    if (f) std::fclose(f);
    return v;
}

int main(int argc, char** argv) {
    std::string dump, run;
    std::vector<double> pv, fields;
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        if (a.compare(0, 7, "--dump=") == 0) dump = a.substr(7);
        if (a.compare(0, 9, "--params=") == 0) {
            std::stringstream ss(a.substr(9));
            std::string item;
            while (std::getline(ss, item, ',')) pv.push_back(std::atof(item.c_str()));
        }
        if (a.compare(0, 9, "--fields=") == 0) fields = read_doubles(a.substr(9));
        if (a.compare(0, 6, "--run=") == 0) run = a.substr(6);
    }
    (void)fields;
    try {
        ScaFES::Parameters params(argc, argv);
        ScaFES::GridGlobal<3> gg(params);
#if PROBLEM == 9
        static const char* NAMES[] = {"RHO", "C", "K", "Q_BRAIN", "Q_TUMOR", "RHO_B", "C_PB", "OMEGA_B_BRAIN",
                                      "OMEGA_B_TUMOR", "T_I", "H", "T_INF", "Q_BC", "DIAMETER", "DEPTH", "T_A"};
        boost::property_tree::ptree pt;
        for (int i = 0; i < 16; ++i) pt.put(std::string("Parameters.") + NAMES[i], pv.at(i));
        TumorHeatEqnFDM<double, 3> ppp(params, gg, false, {"T"}, {1}, {false}, pt, {0}, {0.0},
                                       std::vector<ScaFES::WriteHowOften>(1, ScaFES::WriteHowOften::NEVER), {true},
                                       std::vector<double>(), {false});
#elif PROBLEM == 11
        const std::vector<std::string> names{"F1", "F2", "F3", "G1", "G2", "G3", "U1", "U2", "U3", "V1", "V2", "V3"};
        std::vector<bool> known(12, false);
        for (int i = 0; i < 6; ++i) known[i] = true;
        Latest<LameNavierEqnFDMFirstOrder<double, 3>> ppp(
            params, gg, false, names, std::vector<int>{0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 1, 1}, known,
            std::vector<int>(12, 0), std::vector<double>(12, 0.0),
            std::vector<ScaFES::WriteHowOften>(12, ScaFES::WriteHowOften::NEVER), std::vector<bool>(12, false),
            std::vector<double>());
#elif PROBLEM == 10
        static const char* NAMES[] = {"H", "T_INF", "Q_BC", "Q_SKULL", "EPSILON"};
        boost::property_tree::ptree pt;
        for (int i = 0; i < 5; ++i) pt.put(std::string("Parameters.") + NAMES[i], pv.at(i));
        std::vector<double> dv(10, 0.0);
        dv[9] = pv.at(5);
        std::vector<bool> known(10, true);
        known[9] = false;
        MriFilled ppp(params, gg, false,
                      {"rho", "c", "lambda", "rho_blood", "c_blood", "omega", "T_blood", "q", "surface", "T"},
                      std::vector<int>{0, 0, 0, 0, 0, 0, 0, 0, 0, 1}, known, pt, std::vector<int>(10, 0), dv,
                      std::vector<ScaFES::WriteHowOften>(10, ScaFES::WriteHowOften::NEVER), std::vector<bool>(10, false),
                      std::vector<double>(), std::vector<bool>(10, false));
        ppp.setFields(fields);
#else
#if PROBLEM == 3 || PROBLEM == 5
        std::vector<std::string> names{"A"};
        std::vector<int> sw{1};
        std::vector<bool> known{false};
        std::vector<bool> ce{true};
#else
        std::vector<std::string> names{"F", "G", "U"};
        std::vector<int> sw{0, 0, 1};
        std::vector<bool> known{true, true, false};
        std::vector<bool> ce{false, false, true};
#endif
        const std::size_t nf = names.size();
        CLASS<double, 3> ppp(params, gg, false, names, sw, known, std::vector<int>(nf, 0),
                             std::vector<double>(nf, 0.0),
                             std::vector<ScaFES::WriteHowOften>(nf, ScaFES::WriteHowOften::NEVER), ce,
                             std::vector<double>());
#endif
        if (!dump.empty()) ppp.dumpDeviceForm(dump);
        std::cout << "FORM " << ppp.deviceForm() << std::endl;
#if PROBLEM == 11
        if (!run.empty()) {
            ppp.iterateOverTime();
            const auto& g = ppp.globalGrid().discreteDomain();
            std::vector<double> v;
            for (const auto& df : ppp.latest())
                for (long long m = 0; m < g.nNodesTotal(); ++m) v.push_back(df(g.idxNodeScalar2TupleStyleFortran(m)));
            FILE* f = std::fopen(run.c_str(), "wb");
            if (!f || std::fwrite(v.data(), sizeof(double), v.size(), f) != v.size()) return 4;
            std::fclose(f);
            std::cout << "RAN " << ppp.gpuMilliseconds() << " ms" << std::endl;
        }
#endif
    } catch (const std::exception& e) {
        std::cout << "REFUSED " << e.what() << std::endl;
    }
    return 0;
}
