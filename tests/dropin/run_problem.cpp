// Runs one problem of problems.hpp through the drop-in ScaFES::Problem
// (test infrastructure).  Usage:
//   run_problem <heat_lin|pennes_lin|mirror_pow2|heat_sine|heat_neumann|heat_cauchy> out.bin
//               [--extract-only] [ScaFES options...]
// Writes the final iterate as raw doubles (x fastest); with --extract-only
// prints the device form of the update instead (no GPU needed).
#include <cstdio>
#include <cstring>
#include <iostream>
#include <string>

#include "problems.hpp"

template <class P>
int run(P& ppp, const std::string& out, bool extract) {
    if (extract) {
        std::cout << "FORM " << ppp.deviceForm() << std::endl;
        return 0;
    }
    ppp.iterateOverTime();
    const auto& df = ppp.latest()[0];
    const auto& g = ppp.globalGrid().discreteDomain();
    std::vector<double> v((std::size_t)g.nNodesTotal());
    for (long long m = 0; m < g.nNodesTotal(); ++m) v[m] = df(g.idxNodeScalar2TupleStyleFortran(m));
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
        if (!std::strcmp(argv[i], "--extract-only")) extract = true;
        if (!std::strcmp(argv[i], "--write-like-cl")) write_cl = true;  // U written per --nSnapshots
    }
    try {
        ScaFES::Parameters params(argc, argv);
        ScaFES::GridGlobal<3> gg(params);
        std::vector<ScaFES::WriteHowOften> wr(3, ScaFES::WriteHowOften::NEVER);
        if (write_cl) wr[2] = ScaFES::WriteHowOften::LIKE_GIVEN_AT_CL;
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
