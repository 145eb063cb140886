// Compiles one of the reference's own system-test problem classes,
// unchanged, against the drop-in headers and prints the device form its
// update maps to (test infrastructure; built only where the reference
// checkout is present).  PROBLEM selects the class and the field set of
// the matching reference main3D.cpp:
//   1 HeatEqnFDM/Dirichlet/TimeLinSpaceLin        2 PennesBioheatEqnFDM/Dirichlet/TimeLinSpaceLin
//   3 HeatEqnFdmStencilWidthOne                   4 HeatEqnFDM/Neumann/TimeLinSpaceLin
//   5 PropagationFromLeftLowerCorner              6 HeatEqnFDM/Cauchy/TimeLinSpaceLin
//   7 PennesBioheatEqnFDM/Neumann/TimeLinSpaceLin 8 PennesBioheatEqnFDM/Radiation/TimeLinSpaceLin
#include <iostream>
#include <string>
#include <vector>

#include "ScaFES.hpp"
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

int main(int argc, char** argv) {
    try {
        ScaFES::Parameters params(argc, argv);
        ScaFES::GridGlobal<3> gg(params);
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
        std::cout << "FORM " << ppp.deviceForm() << std::endl;
    } catch (const std::exception& e) {
        std::cout << "REFUSED " << e.what() << std::endl;
    }
    return 0;
}
