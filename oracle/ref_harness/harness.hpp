// Harness shared by the reference-driver programs in oracle/ref_harness/.
//
// These programs compile the UNMODIFIED reference headers (src/ and the
// system-test problem classes under tests/system/) and run the reference's
// own Problem::iterateOverTime() on a configuration given on the command
// line, then dump the final iterate(s) as raw doubles (Fortran order, x
// fastest, no ghost layer).  They are test infrastructure: they generate the
// golden vectors the CPU oracle and the CUDA path are checked against.
//
// Without Boost the reference's Parameters ignores argv and hard-codes a
// 32^DIM grid with one time step (src/ScaFES_Parameters.hpp:1066-1076), so
// the private members are set here through the standard explicit-
// instantiation access rule ([temp.explicit]: access checking does not apply
// to names in explicit instantiations).
#pragma once

#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "ScaFES.hpp"

namespace harness {

template <typename Tag, typename Tag::type M>
struct Grant {
    friend typename Tag::type get(Tag) { return M; }
};

#define HARNESS_MEMBER(NAME, TYPE)                                    \
    struct NAME##Tag {                                                \
        typedef TYPE ScaFES::Parameters::*type;                       \
        friend type get(NAME##Tag);                                   \
    };                                                                \
    template struct Grant<NAME##Tag, &ScaFES::Parameters::NAME>;

HARNESS_MEMBER(mNnodes, std::vector<int>)
HARNESS_MEMBER(mCoordNodeFirst, std::vector<double>)
HARNESS_MEMBER(mCoordNodeLast, std::vector<double>)
HARNESS_MEMBER(mNpartitions, std::vector<int>)
HARNESS_MEMBER(mTau, double)
HARNESS_MEMBER(mNtimesteps, int)
HARNESS_MEMBER(mTimeIntervalStart, double)
HARNESS_MEMBER(mTimeIntervalEnd, double)
HARNESS_MEMBER(mNlayersAtBorder, int)
HARNESS_MEMBER(gOutputLevelMax, int)
HARNESS_MEMBER(gOutputLevelCurr, int)

#define HARNESS_SET(P, NAME) ((P).*get(NAME##Tag()))

struct Config {
    int n[3] = {8, 8, 8};
    double first[3] = {0, 0, 0};
    double last[3] = {1, 1, 1};
    int nsteps = 1;
    double t_start = 0.0;
    double t_end = 1.0;
    double tau = 0.0;  // 0 => (t_end - t_start)/nsteps, as the reference CLI
    std::string out;
    std::string in;
};

// argv: nx ny nz nsteps t_start t_end tau firstx firsty firstz lastx lasty lastz out [in]
inline Config parse(int argc, char** argv) {
    if (argc < 15) {
        std::fprintf(stderr,
                     "usage: %s nx ny nz nsteps t_start t_end tau fx fy fz lx ly lz out.bin [in.bin]\n",
                     argv[0]);
        std::exit(2);
    }
    Config c;
    for (int p = 0; p < 3; ++p) c.n[p] = std::atoi(argv[1 + p]);
    c.nsteps = std::atoi(argv[4]);
    c.t_start = std::atof(argv[5]);
    c.t_end = std::atof(argv[6]);
    c.tau = std::atof(argv[7]);
    for (int p = 0; p < 3; ++p) c.first[p] = std::atof(argv[8 + p]);
    for (int p = 0; p < 3; ++p) c.last[p] = std::atof(argv[11 + p]);
    c.out = argv[14];
    if (argc > 15) c.in = argv[15];
    return c;
}

inline void apply(ScaFES::Parameters& p, const Config& c, int dim) {
    for (int d = 0; d < dim; ++d) {
        HARNESS_SET(p, mNnodes)[d] = c.n[d];
        HARNESS_SET(p, mCoordNodeFirst)[d] = c.first[d];
        HARNESS_SET(p, mCoordNodeLast)[d] = c.last[d];
        HARNESS_SET(p, mNpartitions)[d] = 1;
    }
    HARNESS_SET(p, mNtimesteps) = c.nsteps;
    HARNESS_SET(p, mTimeIntervalStart) = c.t_start;
    HARNESS_SET(p, mTimeIntervalEnd) = c.t_end;
    // src/ScaFES_Parameters.hpp:789 (tau from the interval when not given).
    HARNESS_SET(p, mTau) = (c.tau > 0.0) ? c.tau : (c.t_end - c.t_start) / c.nsteps;
    // nLayersAtBorder: 1 (the reference default) unless HARNESS_NLAYERS says otherwise.
    const char* nl = std::getenv("HARNESS_NLAYERS");
    HARNESS_SET(p, mNlayersAtBorder) = nl ? std::atoi(nl) : 1;
    HARNESS_SET(p, gOutputLevelMax) = 0;
    HARNESS_SET(p, gOutputLevelCurr) = 0;
}

inline std::vector<double> read_raw(const std::string& path, size_t n) {
    std::vector<double> v(n);
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f || std::fread(v.data(), sizeof(double), n, f) != n) {
        std::fprintf(stderr, "cannot read %zu doubles from %s\n", n, path.c_str());
        std::exit(3);
    }
    std::fclose(f);
    return v;
}

// Appends the nodes of a DIM-dimensional data field (Fortran order) to out.
template <typename CT, std::size_t DIM>
void collect(const ScaFES::DataField<CT, DIM>& df, const Config& c, std::vector<double>& out) {
    const int nz = DIM > 2 ? c.n[2] : 1, ny = DIM > 1 ? c.n[1] : 1, nx = c.n[0];
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                ScaFES::Ntuple<int, DIM> n;
                n[0] = i;
                if (DIM > 1) n[1] = j;
                if (DIM > 2) n[2] = k;
                out.push_back(df(n));
            }
}

inline void write_raw(const std::string& path, const std::vector<double>& v) {
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f || std::fwrite(v.data(), sizeof(double), v.size(), f) != v.size()) {
        std::fprintf(stderr, "cannot write %s\n", path.c_str());
        std::exit(4);
    }
    std::fclose(f);
}

}  // namespace harness

// Gives a harness access to the latest iterate of a reference problem
// class: after iterateOverTime() the final swap leaves it in the "old" set
// (src/ScaFES_Problem.hpp:2634-2635).
#define HARNESS_EXPOSE_LATEST(CLASS, CT, DIM)                                      \
    struct CLASS##Latest : public CLASS {                                          \
        using CLASS::CLASS;                                                        \
        const std::vector<ScaFES::DataField<CT, DIM>>& latest() const {            \
            return this->mVectUnknownDfsDomOld;                                    \
        }                                                                          \
    };
