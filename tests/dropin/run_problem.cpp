// Runs one problem of problems.hpp through the drop-in ScaFES::Problem
// (test infrastructure).  Usage:
//   run_problem <heat_lin|pennes_lin|mirror_pow2|heat_sine|heat_neumann|heat_cauchy|
//                pennes_radiation|tumour|mri|yee|yee_varying|lame_first_order> out.bin
//               [--extract-only] [--dump=PATH] [--params=a,b,...] [--fields=PATH]
//               [ScaFES options...]
// Writes the final iterate as raw doubles (x fastest); with --extract-only
// prints the device form of the update instead, with --dump=PATH also
// writes it to PATH (neither needs a GPU).  --params: the tumour's 16
// constants, or the MRI example's H T_INF Q_BC Q_SKULL EPSILON T_INIT;
// --fields: the MRI example's nine known fields, or the Yee cavity's six
// initial fields, raw FP64.  The final iterate holds every unknown field,
// one after the other.
#include <cstdio>
#include <cstring>
#include <iostream>
#include <sstream>
#include <stdexcept>
#include <vector>
#include <string>

#include "problems.hpp"

// Options of the tissue problems and of the device-form dump.
static std::string g_dump;
static std::vector<double> g_params, g_fields;

static std::vector<double> read_doubles(const std::string& path) {
    std::vector<double> v;
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) throw std::runtime_error("cannot read " + path);
    double x;
    while (std::fread(&x, sizeof(double), 1, f) == 1) v.push_back(x);
    std::fclose(f);
    return v;
}

template <class P>
int run(P& ppp, const std::string& out, bool extract) {
    if (!g_dump.empty()) {
        ppp.dumpDeviceForm(g_dump);
        std::cout << "FORM " << ppp.deviceForm() << std::endl;
        return 0;
    }
    if (extract) {
        std::cout << "FORM " << ppp.deviceForm() << std::endl;
        return 0;
    }
    ppp.iterateOverTime();
    const auto& g = ppp.globalGrid().discreteDomain();
    const long long nn = g.nNodesTotal();
    std::vector<double> v;
    for (const auto& df : ppp.latest())
        for (long long m = 0; m < nn; ++m) v.push_back(df(g.idxNodeScalar2TupleStyleFortran(m)));
    FILE* f = std::fopen(out.c_str(), "wb");
    if (!f || std::fwrite(v.data(), sizeof(double), v.size(), f) != v.size()) return 4;
    std::fclose(f);
    std::cout << "GPU_MS " << ppp.gpuMilliseconds() << std::endl;
    return 0;
}

int main(int argc, char** argv) {
    if (argc < 3) return 2;
    const std::string which = argv[1], out = argv[2];
    bool extract = false, write_cl = false;
    for (int i = 3; i < argc; ++i) {
        const std::string a = argv[i];
        if (a == "--extract-only") extract = true;
        if (a == "--write-like-cl") write_cl = true;  // U written per --nSnapshots
        if (a.compare(0, 7, "--dump=") == 0) g_dump = a.substr(7);  // device form to a file, no GPU
        if (a.compare(0, 9, "--params=") == 0) {                      // comma-separated constants
            std::stringstream ss(a.substr(9));
            std::string item;
            while (std::getline(ss, item, ',')) g_params.push_back(std::atof(item.c_str()));
        }
        if (a.compare(0, 9, "--fields=") == 0) g_fields = read_doubles(a.substr(9));  // known fields, raw FP64
    }
    try {
        ScaFES::Parameters params(argc, argv);
        ScaFES::GridGlobal<3> gg(params);
        std::vector<ScaFES::WriteHowOften> wr(3, ScaFES::WriteHowOften::NEVER);
        if (write_cl) wr[2] = ScaFES::WriteHowOften::LIKE_GIVEN_AT_CL;
        if (which == "tumour") {
            TissueTumour<double, 3> p(params, gg, false, {"T"}, {1}, {false}, {0}, {0.0},
                                      std::vector<ScaFES::WriteHowOften>(1, ScaFES::WriteHowOften::NEVER), {true});
            p.setParams(g_params);
            return run(p, out, extract);
        }
        if (which == "mri") {
            std::vector<double> dv(10, 0.0);
            dv[9] = g_params.size() > 5 ? g_params[5] : 0.0;  // initial temperature
            std::vector<bool> known(10, true);
            known[9] = false;
            TissueMri<double, 3> p(params, gg, false,
                                   {"rho", "c", "lambda", "rho_blood", "c_blood", "omega", "T_blood", "q", "surface", "T"},
                                   std::vector<int>{0, 0, 0, 0, 0, 0, 0, 0, 0, 1}, known, std::vector<int>(10, 0), dv,
                                   std::vector<ScaFES::WriteHowOften>(10, ScaFES::WriteHowOften::NEVER),
                                   std::vector<bool>(10, false));
            p.setParams(g_params);
            p.setFields(g_fields);
            return run(p, out, extract);
        }
        if (which == "yee" || which == "yee_varying") {
            YeeCavity<double, 3> p(params, gg, true, {"Ex", "Ey", "Ez", "Hx", "Hy", "Hz"},
                                   std::vector<int>(6, 1), std::vector<bool>(6, false), std::vector<int>(6, 0),
                                   std::vector<double>(6, 0.0),
                                   std::vector<ScaFES::WriteHowOften>(6, ScaFES::WriteHowOften::NEVER),
                                   std::vector<bool>(6, false));
            p.setFields(g_fields);
            p.setVarying(which == "yee_varying");
            return run(p, out, extract);
        }
        if (which == "lame_first_order") {
            std::vector<bool> known(12, false);
            for (int i = 0; i < 6; ++i) known[i] = true;
            LameFirstOrder<double, 3> p(params, gg, false,
                                        {"F1", "F2", "F3", "G1", "G2", "G3", "U1", "U2", "U3", "V1", "V2", "V3"},
                                        std::vector<int>{0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 1, 1}, known,
                                        std::vector<int>(12, 0), std::vector<double>(12, 0.0),
                                        std::vector<ScaFES::WriteHowOften>(12, ScaFES::WriteHowOften::NEVER),
                                        std::vector<bool>(12, false));
            return run(p, out, extract);
        }
        if (which == "mirror_pow2") {
            MirrorPow2<double, 3> p(params, gg, false, {"A"}, {1}, {false}, {0}, {0.0},
                                    std::vector<ScaFES::WriteHowOften>(1, ScaFES::WriteHowOften::NEVER), {true});
            return run(p, out, extract);
        }
        const std::vector<std::string> names{"F", "G", "U"};
        const std::vector<int> sw{0, 0, 1};
        const std::vector<bool> known{true, true, false};
        if (which == "heat_lin") {
            HeatLin<double, 3> p(params, gg, false, names, sw, known, {0, 0, 0}, {0, 0, 0}, wr, {false, false, true});
            return run(p, out, extract);
        }
        if (which == "heat_neumann") {
            HeatFlux<double, 3, 0> p(params, gg, false, names, sw, known, {0, 0, 0}, {0, 0, 0}, wr, {false, false, true});
            return run(p, out, extract);
        }
        if (which == "heat_cauchy") {
            HeatFlux<double, 3, 1> p(params, gg, false, names, sw, known, {0, 0, 0}, {0, 0, 0}, wr, {false, false, true});
            return run(p, out, extract);
        }
        if (which == "pennes_radiation") {
            PennesRadiation<double, 3> p(params, gg, false, names, sw, known, {0, 0, 0}, {0, 0, 0}, wr,
                                         {false, false, true});
            return run(p, out, extract);
        }
        if (which == "pennes_lin") {
            PennesLin<double, 3> p(params, gg, false, names, sw, known, {0, 0, 0}, {0, 0, 0}, wr, {false, false, true});
            return run(p, out, extract);
        }
        if (which == "heat_sine") {
            HeatSine<double, 3> p(params, gg, false, {"F", "U"}, {0, 1}, {true, false}, {0, 0}, {0, 0},
                                  std::vector<ScaFES::WriteHowOften>(2, ScaFES::WriteHowOften::NEVER), {false, false});
            return run(p, out, extract);
        }
    } catch (const std::exception& e) {
        std::cerr << "ERROR " << e.what() << std::endl;
        return 3;
    }
    return 2;
}
