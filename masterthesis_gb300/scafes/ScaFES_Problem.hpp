// ScaFES::Problem -- drop-in CRTP base whose time loop runs on the GPU.
//
// Same constructor, callback names and signatures and accessors as the
// reference's Problem<OWNPRBLM, CT, DIM> (src/ScaFES_Problem.hpp:313-324,
// 433-449, 2418-2553), so a user problem class derived from it compiles
// unchanged.  iterateOverTime() (reference :2559-2715) does:
//
//  1. evaluate the user's evalInner/evalBorder at time steps 0, 1, 2 on the
//     host and store every known field affine in time, K = K_A + time*K_B
//     (checked at step 2); this replaces the per-step evalKnownDfs
//     (:3434-3485);
//  2. run initInner/initBorder on the host for the initial iterate
//     (evalInitPbPhase, :2755-2826);
//  3. extract the update: updateInner<gpu::Sym> at every inner node and
//     updateBorder<gpu::Sym> at every global-border node, at two time
//     steps, give linear forms that must match one of the device kernels --
//     the 7-point star with a source, with constant coefficients or with a
//     centre weight and axis scale per node (the tissue examples), and the
//     Dirichlet, StencilWidthOne mirror, per-class table or per-node border
//     -- or, for a problem with several unknown fields or a leapfrog second
//     phase (updateInner2/updateBorder2), a linear multi-field rule per
//     phase, field and node class (scafes_lin_*); otherwise iterateOverTime
//     throws with the reason (there is no CPU fallback);
//  4. upload, run all nTimesteps sweeps on the device through the C ABI
//     (include/scafes_gb300.h), download the final iterate into the
//     unknown data fields, and compute the max-norm error against the exact
//     solution at the final step for fields with computeError set
//     (DataField::compErrLinf, src/ScaFES_DataField.hpp:1440-1530).
//
// After the run the latest iterate is in mVectUnknownDfsDomOld, as after the
// reference's final pointer swap (:2634-2635).
#ifndef SCAFES_GB300_PROBLEM_HPP
#define SCAFES_GB300_PROBLEM_HPP

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <iostream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "ScaFES_DataField.hpp"
#include "ScaFES_Grid.hpp"
#include "ScaFES_Ntuple.hpp"
#include "ScaFES_Parameters.hpp"
#include "ScaFES_Sym.hpp"
#include "scafes_gb300.h"

namespace ScaFES {

template <class OWNPRBLM, typename CT = double, std::size_t DIM = 3>
class Problem {
public:
    typedef CT value_type;
    template <typename TT>
    using ScaFES_VectDf = std::vector<ScaFES::DataField<TT, DIM>>;
    typedef ScaFES::Ntuple<int, DIM> ScaFES_IntNtuple;

    Problem(const ScaFES::Parameters& params, const ScaFES::GridGlobal<DIM>& gg, const bool& useLeapfrog,
            const std::vector<std::string>& nameDatafield, const std::vector<int>& stencilWidth,
            const std::vector<bool>& isKnownDf, const std::vector<int>& nLayers = std::vector<int>(),
            const std::vector<CT>& defaultValue = std::vector<CT>(),
            const std::vector<ScaFES::WriteHowOften>& writeToFile = std::vector<ScaFES::WriteHowOften>(),
            const std::vector<bool>& computeError = std::vector<bool>(),
            const std::vector<CT>& geomparamsInit = std::vector<CT>(),
            const std::vector<bool>& checkConvergence = std::vector<bool>())
        : mParams(params), mGG(gg), mUseLeapfrog(useLeapfrog), mNames(nameDatafield),
          mStencilWidth(stencilWidth), mIsKnown(isKnownDf), mComputeError(computeError),
          mVectParamsCurr(geomparamsInit), mWriteToFile(writeToFile) {
        (void)nLayers; (void)checkConvergence;
        // Argument checks of the reference constructor (:1400-1423).
        const std::size_t nf = nameDatafield.size();
        if (nf == 0 || stencilWidth.size() != nf || isKnownDf.size() != nf)
            throw std::runtime_error("ScaFES::Problem: field name, stencil width and isKnownDf vectors differ in size");
        if (!computeError.empty() && computeError.size() != nf)
            throw std::runtime_error("ScaFES::Problem: computeError must have one entry per field");
        if (DIM != 3) throw std::runtime_error("ScaFES::Problem: the GPU engine runs DIM = 3 problems");
        mComputeError.resize(nf, false);
        mN = gg.discreteDomain().nNodesTotal();
        for (std::size_t f = 0; f < nf; ++f) {
            if (!isKnownDf[f]) mUnknownIdx.push_back((int)f);
        }
        if (mUnknownIdx.empty()) throw std::runtime_error("ScaFES::Problem: no unknown data field");
        const std::size_t nu = mUnknownIdx.size();
        mKnownNewStore.assign(nf * mN, CT());
        mKnownOldStore.assign(nf * mN, CT());
        mUnknownNewStore.assign(nu * mN, CT());
        mUnknownOldStore.assign(nu * mN, CT());
        for (std::size_t f = 0; f < nf; ++f) {
            mVectKnownDfsDomNew.emplace_back(nameDatafield[f], &mGG, mKnownNewStore.data() + f * mN, stencilWidth[f]);
            mVectKnownDfsDomOld.emplace_back(nameDatafield[f], &mGG, mKnownOldStore.data() + f * mN, stencilWidth[f]);
        }
        // Each unknown field starts at its default value, which the init
        // callbacks then overwrite where they write (the reference resets
        // the unknown fields to defaultValue before evalInitPbPhase,
        // src/ScaFES_Problem.hpp:2999-3027, 2623).
        for (std::size_t u = 0; u < nu; ++u) {
            const int f = mUnknownIdx[u];
            if ((std::size_t)f < defaultValue.size())
                std::fill(mUnknownNewStore.begin() + u * mN, mUnknownNewStore.begin() + (u + 1) * mN, defaultValue[f]);
        }
        for (std::size_t u = 0; u < nu; ++u) {
            const int f = mUnknownIdx[u];
            mVectUnknownDfsDomNew.emplace_back(nameDatafield[f], &mGG, mUnknownNewStore.data() + u * mN, stencilWidth[f]);
            mVectUnknownDfsDomOld.emplace_back(nameDatafield[f], &mGG, mUnknownOldStore.data() + u * mN, stencilWidth[f]);
        }
    }

    Problem(const Problem&) = delete;
    Problem& operator=(const Problem&) = delete;
    virtual ~Problem() {
        if (mHandle) scafes_gpu_destroy(mHandle);
    }

    // ---- accessors of the reference interface (:2418-2553) -----------------
    const ScaFES::Parameters& params() const { return mParams; }
    const double& gridsize(const int& idx) const { return mGG.discreteDomain().gridsize(idx); }
    const double& tau() const { return mParams.tau(); }
    const int& nTimesteps() const { return mParams.nTimesteps(); }
    const ScaFES::GridGlobal<DIM>& globalGrid() const { return mGG; }
    const ScaFES_IntNtuple& nNodes() const { return mGG.discreteDomain().nNodes(); }
    const int& nNodes(const int& dim) const { return mGG.discreteDomain().nNodes(dim); }
    ScaFES::Ntuple<double, DIM> coordinates(const ScaFES_IntNtuple& n) const {
        return mGG.discreteDomain().coordinates(n);
    }
    double time(const int& timestep) const { return mParams.timeIntervalStart() + timestep * mParams.tau(); }
    ScaFES_IntNtuple connect(const ScaFES_IntNtuple& n, const int& dir) { return mGG.discreteDomain().neigh(n, dir); }
    const std::vector<CT>& vectParamsCurr() const { return mVectParamsCurr; }
    gpu::Known knownDf(const int& idx, const ScaFES_IntNtuple& n) const { return knownDfNew(idx, n); }
    gpu::Known knownDfNew(const int& idx, const ScaFES_IntNtuple& n) const {
        return gpu::Known((double)mVectKnownDfsDomNew[idx](n), gpu::Sym::known(idx, 0));
    }
    gpu::Known knownDfOld(const int& idx, const ScaFES_IntNtuple& n) const {
        return gpu::Known((double)mVectKnownDfsDomOld[idx](n), gpu::Sym::known(idx, 1));
    }
    const ScaFES_VectDf<CT>& vectSol() const { return mVectKnownDfsDomNew; }

    // ---- results of the last iterateOverTime -------------------------------
    double errLinf(int field) const {
        auto it = mErrLinf.find(field);
        return it == mErrLinf.end() ? -1.0 : it->second;
    }
    double gpuMilliseconds() const { return mGpuMs; }
    const std::string& gpuKernelSummary() const { return mSummary; }

    void iterateOverTime();

    // Runs the host part of iterateOverTime (known fields, initial iterate,
    // stencil extraction) without touching the GPU and returns the device
    // form the update maps to; throws if it maps to none.
    const std::string& deviceForm() {
        prepareDevice();
        return mSummary;
    }

    // Runs the same host part and writes everything the device run would
    // receive -- the configuration, the border rules and every field it
    // uploads except the initial iterate -- to `path` as named FP64
    // arrays (16-byte name, int64 count, values).  Two problem classes
    // whose files are equal byte for byte run the same device computation.
    void dumpDeviceForm(const std::string& path) {
        prepareDevice();
        FILE* f = std::fopen(path.c_str(), "wb");
        if (!f) throw std::runtime_error("ScaFES::Problem: cannot write " + path);
        auto put = [&](const char* name, const double* v, long long n) {
            char tag[16] = {};
            std::strncpy(tag, name, sizeof(tag) - 1);
            std::fwrite(tag, 1, sizeof(tag), f);
            std::fwrite(&n, sizeof(n), 1, f);
            if (n > 0) std::fwrite(v, sizeof(double), (std::size_t)n, f);
        };
        if (mLinear) {
            // Multi-field rules: per (phase, field, class) the term count,
            // the constant and (src, dx, dy, dz, w) per term.
            std::vector<double> r;
            for (std::size_t s = 0; s < mLinTerms.size(); ++s) {
                r.push_back((double)mLinTerms[s].size());
                r.push_back(mLinCst[s]);
                for (const auto& t : mLinTerms[s]) {
                    const double q[5] = {(double)t.src, (double)t.dx, (double)t.dy, (double)t.dz, t.w};
                    r.insert(r.end(), q, q + 5);
                }
            }
            const Grid<DIM>& g = mGG.discreteDomain();
            const double cfgv[] = {(double)g.nNodes(0), (double)g.nNodes(1), (double)g.nNodes(2),
                                   (double)mUnknownIdx.size(), (double)mLinPhases};
            put("lin_cfg", cfgv, 5);
            put("lin_rules", r.data(), (long long)r.size());
            if (std::fclose(f) != 0) throw std::runtime_error("ScaFES::Problem: cannot write " + path);
            return;
        }
        const scafes_cfg& c = mCfg;
        const double cfgv[] = {(double)c.n_nodes[0], (double)c.n_nodes[1], (double)c.n_nodes[2],
                               c.coord_first[0], c.coord_first[1], c.coord_first[2],
                               c.coord_last[0], c.coord_last[1], c.coord_last[2], c.tau, c.t_start,
                               (double)c.n_layers_at_border, (double)c.precision, (double)c.border,
                               c.c0, c.cp[0], c.cp[1], c.cp[2], c.cf, mGcenter, mGrate, mGpoly ? 1.0 : 0.0};
        put("cfg", cfgv, (long long)(sizeof(cfgv) / sizeof(double)));
        if (c.border == SCAFES_BORDER_TABLE)
            put("forms", &mForms[0].cu, (long long)(sizeof(mForms) / sizeof(double)));
        put("F_A", mFa.data(), (long long)mFa.size());
        put("F_B", mFb.data(), (long long)mFb.size());
        put("G_A", mGa.data(), (long long)mGa.size());
        put("G_B", mGb.data(), (long long)mGb.size());
        for (int k = 0; k < 3; ++k) put(k == 0 ? "G_C" : k == 1 ? "G_D" : "G_E", mGhi[k].data(), (long long)mGhi[k].size());
        put("C0", mC0.data(), (long long)mC0.size());
        put("CA", mCA.data(), (long long)mCA.size());
        put("node_rules", mNodeRules.empty() ? nullptr : &mNodeRules[0].cu, (long long)mNodeRules.size() * 8);
        if (std::fclose(f) != 0) throw std::runtime_error("ScaFES::Problem: cannot write " + path);
    }

protected:
    ScaFES::Parameters mParams;
    const ScaFES::GridGlobal<DIM>& mGG;
    bool mUseLeapfrog;
    std::vector<std::string> mNames;
    std::vector<int> mStencilWidth;
    std::vector<bool> mIsKnown;
    std::vector<bool> mComputeError;
    std::vector<CT> mVectParamsCurr;
    std::vector<int> mUnknownIdx;
    long long mN = 0;
    std::vector<CT> mKnownNewStore, mKnownOldStore, mUnknownNewStore, mUnknownOldStore;
    ScaFES_VectDf<CT> mVectKnownDfsDomNew, mVectKnownDfsDomOld;
    ScaFES_VectDf<CT> mVectUnknownDfsDomNew, mVectUnknownDfsDomOld;
    std::map<std::string, double> mWallClockTimes;

private:
    struct Affine { std::vector<double> a, b; bool zero = true, timed = false; };
    struct Form {
        double c0 = 0, cp[3] = {0, 0, 0}, cst = 0;
        std::map<std::pair<int, int>, double> known;  // (field, when) -> coefficient
    };

    bool isBorder(const ScaFES_IntNtuple& n) const {
        const Grid<DIM>& g = mGG.discreteDomain();
        const int L = mParams.nLayersAtBorder();
        for (std::size_t p = 0; p < DIM; ++p)
            if (n[p] < g.idxNodeFirst(p) + L || n[p] > g.idxNodeLast(p) - L) return true;
        return false;
    }

    // Known fields of time step t into the "new" set (evalGlobInner/Border).
    void evalKnownAt(int t) {
        const Grid<DIM>& g = mGG.discreteDomain();
        OWNPRBLM* self = static_cast<OWNPRBLM*>(this);
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
        for (long long m = 0; m < mN; ++m) {
            const ScaFES_IntNtuple n = g.idxNodeScalar2TupleStyleFortran(m);
            if (isBorder(n)) self->evalBorder(mVectKnownDfsDomNew, n, t);
            else self->evalInner(mVectKnownDfsDomNew, n, t);
        }
    }

    // Records one update callback at node n for time step t.
    template <bool BORDER, int PHASE = 1>
    std::vector<gpu::Sym> record(const ScaFES_IntNtuple& n, int t, std::string& err) {
        gpu::Recorder<DIM> rec;
        rec.centre = n;
        rec.grid = &mGG.discreteDomain();
        const std::size_t nu = mUnknownIdx.size();
        rec.out.resize(nu);
        ScaFES_VectDf<gpu::Sym> vNew, vOld;
        for (std::size_t u = 0; u < nu; ++u) {
            const int f = mUnknownIdx[u];
            vNew.emplace_back(mNames[f], &mGG, &rec, (int)u, true, mStencilWidth[f]);
            vOld.emplace_back(mNames[f], &mGG, &rec, (int)u, false, mStencilWidth[f]);
            // Copy-before-update: a node the callback leaves alone keeps its
            // old value (src/ScaFES_Problem.hpp:5078-5082).
            rec.out[u] = gpu::Sym::unknown((int)u, 0, 0, 0);
        }
        OWNPRBLM* self = static_cast<OWNPRBLM*>(this);
        gpu::comparison_on_unknown() = false;
        gpu::converted_unknown() = false;
        if (PHASE == 2) {
            if (BORDER) self->template updateBorder2<gpu::Sym>(vNew, vOld, n, t);
            else self->template updateInner2<gpu::Sym>(vNew, vOld, n, t);
        } else {
            if (BORDER) self->template updateBorder<gpu::Sym>(vNew, vOld, n, t);
            else self->template updateInner<gpu::Sym>(vNew, vOld, n, t);
        }
        err = rec.error;
        if (err.empty() && gpu::comparison_on_unknown())
            err = "update callback branches on the value of an unknown (not a linear stencil)";
        if (err.empty() && gpu::converted_unknown())
            err = "update callback turns an unknown into a number (not a linear stencil)";
        return rec.out;
    }

    static std::string describe(const gpu::Sym& s) {
        std::ostringstream os;
        os.precision(17);
        os << s.constant();
        for (const auto& kv : s.terms()) {
            const auto& k = kv.first;
            if (k.kind == 0) os << " + " << kv.second << "*U" << k.a << "(" << k.b << "," << k.c << "," << k.d << ")";
            else if (k.kind == 2) os << " + " << kv.second << "*U" << k.a << "(0,0,0)^" << k.b;
            else os << " + " << kv.second << "*K" << k.a << (k.b ? "(old)" : "(new)");
        }
        if (s.bad()) os << " [non-linear]";
        return os.str();
    }

    static bool same(const gpu::Sym& a, const gpu::Sym& b) {
        if (a.bad() || b.bad()) return false;
        if (a.constant() != b.constant() || a.terms().size() != b.terms().size()) return false;
        for (const auto& kv : a.terms()) {
            bool found = false;
            for (const auto& kw : b.terms())
                if (kw.first == kv.first) { found = kw.second == kv.second; break; }
            if (!found) return false;
        }
        return true;
    }

    // The inner form -> 7-point star coefficients + source terms.
    Form starForm(const gpu::Sym& s) const {
        if (s.bad()) throw std::runtime_error("ScaFES::Problem: updateInner is not linear in the unknowns: " + describe(s));
        Form F;
        F.cst = s.constant();
        double cm[3] = {0, 0, 0}, cpp[3] = {0, 0, 0};
        for (const auto& kv : s.terms()) {
            const auto& k = kv.first;
            if (k.kind == 1) { F.known[{k.a, k.b}] += kv.second; continue; }
            if (k.kind == 2) throw std::runtime_error("ScaFES::Problem: updateInner is not linear in the unknowns: " + describe(s));
            if (k.a != 0) throw std::runtime_error("ScaFES::Problem: updateInner couples several unknown fields");
            const int nz = (k.b != 0) + (k.c != 0) + (k.d != 0);
            const int mag = std::abs(k.b) + std::abs(k.c) + std::abs(k.d);
            if (nz == 0) { F.c0 += kv.second; continue; }
            if (nz != 1 || mag != 1)
                throw std::runtime_error("ScaFES::Problem: updateInner reaches beyond the 7-point star: " + describe(s));
            const int p = k.b ? 0 : (k.c ? 1 : 2);
            const int sgn = k.b + k.c + k.d;
            (sgn < 0 ? cm : cpp)[p] += kv.second;
        }
        for (int p = 0; p < 3; ++p) {
            if (cm[p] != cpp[p])
                throw std::runtime_error("ScaFES::Problem: updateInner is not symmetric along an axis: " + describe(s));
            F.cp[p] = cm[p];
        }
        return F;
    }

    // The table rule of one border node's recorded form, or why there is
    // none: u_new = cu*u + sum_d cn[d]*u_d + cf*(the inner source)
    //               + cg_old*G(old) + cg_new*G(new) + cu4*u^4, G one known field.
    std::string tableRule(const gpu::Sym& s1, const gpu::Sym& s2, const Form& F, const std::vector<Affine>& aff,
                          int& gfield, scafes_border_form& r) const {
        if (!same(s1, s2)) return "the rule changes between time steps";
        if (s1.constant() != 0.0) return "a constant term";
        double cf = 0.0;
        bool have_cf = false;
        std::map<std::pair<int, int>, double> src;
        for (const auto& kv : s1.terms()) {
            const auto& k = kv.first;
            if (k.kind == 2) {
                if (k.a != 0) return "several unknown fields";
                if (k.b != 4) return "a power of the node's unknown other than 1 and 4";
                r.cu4 += kv.second;
                continue;
            }
            if (k.kind == 0) {
                if (k.a != 0) return "several unknown fields";
                const int nz = (k.b != 0) + (k.c != 0) + (k.d != 0);
                const int mag = std::abs(k.b) + std::abs(k.c) + std::abs(k.d);
                if (nz == 0) { r.cu += kv.second; continue; }
                if (nz != 1 || mag != 1) return "a neighbour beyond the 7-point star";
                const int p = k.b ? 0 : (k.c ? 1 : 2);
                const int sgn = k.b + k.c + k.d;
                r.cn[2 * p + (sgn > 0 ? 1 : 0)] += kv.second;
                continue;
            }
            if (aff[k.a].zero) continue;  // a known field that is 0 everywhere
            if (F.known.count({k.a, k.b})) { src[{k.a, k.b}] += kv.second; continue; }
            if (gfield == -1) gfield = k.a;
            if (k.a != gfield) return "more than one border known field";
            (k.b ? r.cg_old : r.cg_new) += kv.second;
        }
        // The source terms must be a multiple of the inner update's source.
        for (const auto& kv : F.known) {
            if (aff[kv.first.first].zero) continue;
            const auto it = src.find(kv.first);
            const double c = it == src.end() ? 0.0 : it->second;
            const double ratio = c / kv.second;
            if (!have_cf) { cf = ratio; have_cf = true; }
            else if (ratio != cf) return "source terms that are not a multiple of the inner source";
        }
        r.cf = cf;
        return std::string();
    }

    // The rule of one border node alone (SCAFES_BORDER_NODES):
    //   u_new = cu*u + sum_d cn[d]*u_d + cst,
    // known fields folded into cst with their value at the node (so they must
    // not change in time), or why there is none.
    std::string nodeRule(const gpu::Sym& s1, const gpu::Sym& s2, const std::vector<Affine>& aff, long long m,
                         scafes_border_node_rule& r) const {
        if (!same(s1, s2)) return "the rule changes between time steps";
        r.cst = s1.constant();
        for (const auto& kv : s1.terms()) {
            const auto& k = kv.first;
            if (k.kind == 2) return "a power of the node's unknown";
            if (k.kind == 0) {
                if (k.a != 0) return "several unknown fields";
                const int nz = (k.b != 0) + (k.c != 0) + (k.d != 0);
                const int mag = std::abs(k.b) + std::abs(k.c) + std::abs(k.d);
                if (nz == 0) { r.cu += kv.second; continue; }
                if (nz != 1 || mag != 1) return "a neighbour beyond the 7-point star";
                const int p = k.b ? 0 : (k.c ? 1 : 2);
                r.cn[2 * p + ((k.b + k.c + k.d) > 0 ? 1 : 0)] += kv.second;
                continue;
            }
            const Affine& A = aff[k.a];
            if (A.zero) continue;
            if (A.a.empty() || A.timed) return "a known field that changes in time";
            r.cst += kv.second * A.a[m];
        }
        return std::string();
    }

    void fitAffine(std::vector<Affine>& aff, std::vector<CT>& k0, std::vector<CT>& k1) {
        const std::size_t nf = mNames.size();
        const double t0 = time(0), tau = mParams.tau();
        aff.assign(nf, Affine());
        for (std::size_t f = 0; f < nf; ++f) {
            Affine& A = aff[f];
            A.a.resize(mN);
            A.b.resize(mN);
            for (long long m = 0; m < mN; ++m) {
                const double v0 = (double)k0[f * mN + m], v1 = (double)k1[f * mN + m];
                const double b = tau != 0.0 ? (v1 - v0) / tau : 0.0;
                A.b[m] = b;
                A.a[m] = v0 - t0 * b;
                if (v0 != 0.0 || v1 != 0.0) A.zero = false;
                if (b != 0.0) A.timed = true;
            }
        }
    }

    // Known field f as a polynomial of degree <= 4 in
    //   s = (time(t) - t_center) * t_rate,  s in [-1, 1] over steps 0..T
    // (the device's time basis of G, scafes_gpu_set_border_time_basis):
    // interpolation at five Chebyshev points of the run, rounded to steps,
    // checked at three other steps.  Fills mGa, mGb, mGhi and the basis, or
    // throws if the field is not such a polynomial (to 1e-11 relative).
    void fitTimePolynomial(int f) {
        const int T = mParams.nTimesteps();
        const double ta = time(0), tb = time(T);
        mGcenter = 0.5 * (ta + tb);
        mGrate = tb > ta ? 2.0 / (tb - ta) : 1.0;
        std::vector<int> steps;
        if (T <= 4) {
            for (int k = 0; k <= T; ++k) steps.push_back(k);
        } else {
            const double pi = 3.14159265358979323846;
            for (int j = 0; j < 5; ++j)
                steps.push_back((int)std::lround(0.5 * T * (1.0 - std::cos((2 * j + 1) * pi / 10.0))));
        }
        const int np = (int)steps.size();
        // Inverse of the Vandermonde matrix V[j][k] = s_j^k (Gauss-Jordan,
        // partial pivoting; at most 5 x 5).
        double V[5][10] = {};
        for (int j = 0; j < np; ++j) {
            const double sj = (time(steps[j]) - mGcenter) * mGrate;
            double pw = 1.0;
            for (int k = 0; k < np; ++k, pw *= sj) V[j][k] = pw;
            V[j][np + j] = 1.0;
        }
        for (int c = 0; c < np; ++c) {
            int piv = c;
            for (int r = c + 1; r < np; ++r)
                if (std::fabs(V[r][c]) > std::fabs(V[piv][c])) piv = r;
            if (V[piv][c] == 0.0) throw std::runtime_error("ScaFES::Problem: time samples of a border field coincide");
            for (int k = 0; k < 2 * np; ++k) std::swap(V[c][k], V[piv][k]);
            const double d = V[c][c];
            for (int k = 0; k < 2 * np; ++k) V[c][k] /= d;
            for (int r = 0; r < np; ++r) {
                if (r == c || V[r][c] == 0.0) continue;
                const double q = V[r][c];
                for (int k = 0; k < 2 * np; ++k) V[r][k] -= q * V[c][k];
            }
        }
        std::vector<double> co[5];
        for (int k = 0; k < 5; ++k) co[k].assign((std::size_t)mN, 0.0);
        std::vector<double> vmax((std::size_t)mN, 1.0);
        for (int j = 0; j < np; ++j) {
            evalKnownAt(steps[j]);
            for (long long m = 0; m < mN; ++m) {
                const double v = (double)mKnownNewStore[f * mN + m];
                vmax[m] = std::max(vmax[m], std::fabs(v));
                for (int k = 0; k < np; ++k) co[k][m] += V[k][np + j] * v;
            }
        }
        if (T > 4) {
            for (int t : {1, T / 3, (2 * T) / 3 + 1}) {
                evalKnownAt(t);
                const double st = (time(t) - mGcenter) * mGrate;
                for (long long m = 0; m < mN; ++m) {
                    double p = co[4][m];
                    for (int k = 3; k >= 0; --k) p = std::fma(p, st, co[k][m]);
                    const double v = (double)mKnownNewStore[f * mN + m];
                    if (std::fabs(p - v) > 1e-11 * vmax[m])
                        throw std::runtime_error("ScaFES::Problem: border field " + mNames[f] +
                                                 " is neither affine nor a polynomial of degree <= 4 in time");
                }
            }
        }
        mGa.swap(co[0]);
        mGb.swap(co[1]);
        for (int k = 0; k < 3; ++k) mGhi[k].swap(co[2 + k]);
        mGpoly = true;
    }

    int precisionCode() const {
        const std::string& p = mParams.gpuPrecision();
        if (p == "f64") return SCAFES_PREC_F64;
        if (p == "f32x2") return SCAFES_PREC_F32X2;
        if (p == "f32") return SCAFES_PREC_F32;
        throw std::runtime_error("ScaFES::Problem: unknown --gpuPrecision " + p);
    }

    void check(int rc) const {
        if (rc != SCAFES_OK)
            throw std::runtime_error(std::string("ScaFES::Problem (GPU): ") +
                                     (mHandle ? scafes_gpu_last_error(mHandle) : scafes_last_error()));
    }

    void prepareDevice();
    // Several unknown fields or a leapfrog second phase: the linear
    // multi-field rules of scafes_lin_* (one per phase, field and node class).
    void prepareLinear();
    void runLinear();
    std::string linearRule(const gpu::Sym& s, const std::vector<Affine>& aff, std::vector<scafes_lin_term>& terms,
                           double& cst) const;
    bool mLinear = false;
    int mLinPhases = 1;
    // [phase][field][class] -> terms, constant
    std::vector<std::vector<scafes_lin_term>> mLinTerms;
    std::vector<double> mLinCst;

    // What prepareDevice hands to the device run.
    bool mPrepared = false;
    scafes_cfg mCfg = {};
    std::vector<double> mFa, mFb, mGa, mGb;
    std::vector<double> mC0, mCA;                      // coefficient slots (variable coefficients)
    std::vector<scafes_border_node_rule> mNodeRules;   // per-node border rules
    std::vector<double> mGhi[3];       // G_C .. G_E of a polynomial-in-time border field
    bool mGpoly = false;
    double mGcenter = 0.0, mGrate = 1.0;
    scafes_border_form mForms[SCAFES_BORDER_CLASSES] = {};
    std::vector<ScaFES::WriteHowOften> mWriteToFile;
    std::string mSnapshotFile;
    scafes_handle* mHandle = nullptr;
    std::map<int, double> mErrLinf;
    double mGpuMs = 0.0;
    std::string mSummary;
};

template <class OWNPRBLM, typename CT, std::size_t DIM>
void Problem<OWNPRBLM, CT, DIM>::prepareDevice() {
    using clock = std::chrono::steady_clock;
    if (mPrepared) return;
    if (mUseLeapfrog || mUnknownIdx.size() != 1) {
        prepareLinear();
        return;
    }
    const std::size_t nf = mNames.size();
    const Grid<DIM>& g = mGG.discreteDomain();

    // 1. Known fields at steps 0, 1, 2 -> affine in time.
    auto t_eval = clock::now();
    evalKnownAt(0);
    std::vector<CT> k0 = mKnownNewStore;
    evalKnownAt(1);
    std::vector<CT> k1 = mKnownNewStore;
    std::vector<Affine> aff;
    fitAffine(aff, k0, k1);
    evalKnownAt(2);
    const double t2 = time(2);
    for (std::size_t f = 0; f < nf; ++f) {
        if (!mIsKnown[f]) continue;
        for (long long m = 0; m < mN; ++m) {
            const double pred = aff[f].a[m] + t2 * aff[f].b[m];
            const double v = (double)mKnownNewStore[f * mN + m];
            if (std::fabs(pred - v) > 1e-12 * std::max(1.0, std::fabs(v))) {
                aff[f].timed = true;
                aff[f].zero = false;
                aff[f].a.clear();  // marks "not affine in time"
                break;
            }
        }
    }
    mWallClockTimes["evalKnownDf"] += std::chrono::duration<double>(clock::now() - t_eval).count();

    // 2. Initial iterate (time step 0) on the host: initInner/initBorder,
    // or a snapshot file with --initfile (evalInitPbPhase, :2766-2790,
    // readDfsFromFile :4427).
    auto t_init = clock::now();
    std::copy(k0.begin(), k0.end(), mKnownNewStore.begin());
    mKnownOldStore = k0;
    if (mParams.readInitFile()) {
        int nn[3] = {0, 0, 0}, count = 0;
        const std::string& path = mParams.nameInitFile();
        if (scafes_snapshot_info(path.c_str(), nn, &count) != SCAFES_OK)
            throw std::runtime_error("ScaFES::Problem: cannot read init file " + path + ": " + scafes_last_error());
        for (std::size_t p = 0; p < DIM; ++p)
            if (nn[p] != g.nNodes(p))
                throw std::runtime_error("ScaFES::Problem: init file " + path + " holds another grid");
        int idx = mParams.initFileIndex();
        if (idx < 0) idx += count;
        if (idx < 0 || idx >= count)
            throw std::runtime_error("ScaFES::Problem: init file " + path + " has no snapshot " +
                                     std::to_string(mParams.initFileIndex()));
        std::vector<double> u((std::size_t)mN);
        long long step = 0;
        double t_file = 0.0;
        if (scafes_snapshot_read(path.c_str(), idx, u.data(), u.size(), &step, &t_file) != SCAFES_OK)
            throw std::runtime_error("ScaFES::Problem: cannot read init file " + path + ": " + scafes_last_error());
        for (long long m = 0; m < mN; ++m) mUnknownNewStore[m] = (CT)u[m];
        for (auto& df : mVectUnknownDfsDomNew) df.time() = (CT)time(0);
    } else {
        OWNPRBLM* self = static_cast<OWNPRBLM*>(this);
        for (auto& df : mVectUnknownDfsDomNew) df.time() = (CT)time(0);
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
        for (long long m = 0; m < mN; ++m) {
            const ScaFES_IntNtuple n = g.idxNodeScalar2TupleStyleFortran(m);
            if (isBorder(n)) self->template initBorder<CT>(mVectUnknownDfsDomNew, mVectParamsCurr, n, 0);
            else self->template initInner<CT>(mVectUnknownDfsDomNew, mVectParamsCurr, n, 0);
        }
    }
    mWallClockTimes["init"] += std::chrono::duration<double>(clock::now() - t_init).count();

    // 3. Extract the update (known values of step 1 as "new", step 0 as "old").
    auto t_rec = clock::now();
    std::copy(k1.begin(), k1.end(), mKnownNewStore.begin());
    std::string err;
    // Probe nodes: the inner form must not change between time steps.
    std::vector<ScaFES_IntNtuple> probes;
    {
        ScaFES_IntNtuple lo(1), hi, mid;
        for (std::size_t p = 0; p < DIM; ++p) { hi[p] = g.nNodes(p) - 2; mid[p] = g.nNodes(p) / 2; }
        probes.push_back(mid);
        probes.push_back(lo);
        probes.push_back(hi);
        unsigned s = 12345u;
        for (int k = 0; k < 5; ++k) {
            ScaFES_IntNtuple r;
            for (std::size_t p = 0; p < DIM; ++p) {
                s = s * 1103515245u + 12345u;
                r[p] = 1 + (int)((s >> 8) % (unsigned)(g.nNodes(p) - 2));
            }
            probes.push_back(r);
        }
    }
    for (const auto& n : probes) {
        if (isBorder(n)) continue;
        gpu::Sym s1 = record<false>(n, 1, err)[0];
        if (!err.empty()) throw std::runtime_error("ScaFES::Problem: " + err);
        gpu::Sym s2 = record<false>(n, 2, err)[0];
        if (!err.empty()) throw std::runtime_error("ScaFES::Problem: " + err);
        if (!same(s1, s2))
            throw std::runtime_error("ScaFES::Problem: updateInner changes between time steps: " + describe(s1) +
                                     " vs " + describe(s2));
    }

    // Every inner node at step 1: its 7-point star, and its source
    // F(t_old) = cst + sum_j b_j K_j as F_A + time * F_B.  When every node
    // has the same star the device runs the constant-coefficient sweep; when
    // the coefficients change from node to node (coefficients read from
    // known fields or from the node's coordinates, as in the reference's
    // tissue examples) it runs the variable-coefficient sweep with the
    // per-node centre weight C0 and axis scale CA.
    std::vector<double> fa((std::size_t)mN, 0.0), fb;
    std::vector<double> c0n((std::size_t)mN, 0.0), cpn[3];
    for (int p = 0; p < 3; ++p) cpn[p].assign((std::size_t)mN, 0.0);
    bool any_timed = false;
    for (std::size_t f = 0; f < nf; ++f) any_timed = any_timed || (mIsKnown[f] && aff[f].timed);
    if (any_timed) fb.assign((std::size_t)mN, 0.0);
    Form F0;
    bool have_first = false, uniform = true, has_f = false, has_fb = false;
    std::string inner_err;
    {
        // The first inner node's form is the reference the others compare with.
        for (long long m = 0; m < mN && !have_first; ++m) {
            const ScaFES_IntNtuple n = g.idxNodeScalar2TupleStyleFortran(m);
            if (isBorder(n)) continue;
            gpu::Sym s = record<false>(n, 1, err)[0];
            if (!err.empty()) throw std::runtime_error("ScaFES::Problem: " + err);
            F0 = starForm(s);
            have_first = true;
        }
        if (!have_first) throw std::runtime_error("ScaFES::Problem: the grid has no inner nodes");
    }
#ifdef _OPENMP
#pragma omp parallel for schedule(static) reduction(&& : uniform) reduction(|| : has_f, has_fb)
#endif
    for (long long m = 0; m < mN; ++m) {
        const ScaFES_IntNtuple n = g.idxNodeScalar2TupleStyleFortran(m);
        if (isBorder(n)) continue;
        std::string e;
        Form F;
        try {
            gpu::Sym s = record<false>(n, 1, e)[0];
            if (e.empty()) F = starForm(s);
        } catch (const std::exception& x) {
            e = x.what();
        }
        if (e.empty()) {
            bool same_form = F.c0 == F0.c0 && F.cst == F0.cst && F.known.size() == F0.known.size();
            for (int p = 0; p < 3; ++p) same_form = same_form && F.cp[p] == F0.cp[p];
            c0n[m] = F.c0;
            for (int p = 0; p < 3; ++p) cpn[p][m] = F.cp[p];
            double va = F.cst, vb = 0.0;
            if (F.cst != 0.0) has_f = true;
            for (const auto& kv : F.known) {
                const auto it = F0.known.find(kv.first);
                same_form = same_form && it != F0.known.end() && it->second == kv.second;
                const int j = kv.first.first;
                const Affine& A = aff[j];
                if (A.zero) continue;
                if (A.a.empty()) {
                    e = "known field " + mNames[j] + " is not affine in time; the device path takes affine known fields";
                    break;
                }
                has_f = true;
                const bool is_new = kv.first.second == 0;
                va += kv.second * (A.a[m] + (is_new ? mParams.tau() * A.b[m] : 0.0));
                if (A.timed) {
                    vb += kv.second * A.b[m];
                    has_fb = true;
                }
            }
            fa[m] = va;
            if (!fb.empty()) fb[m] = vb;
            uniform = uniform && same_form;
        }
        if (!e.empty()) {
#ifdef _OPENMP
#pragma omp critical(scafes_inner_error)
#endif
            if (inner_err.empty()) inner_err = e;
        }
    }
    if (!inner_err.empty()) throw std::runtime_error("ScaFES::Problem: " + inner_err);
    // Border rules of the table kind read the inner source at border nodes:
    // with one inner form, its source is defined there as well.
    if (uniform) {
        for (long long m = 0; m < mN; ++m) {
            if (!isBorder(g.idxNodeScalar2TupleStyleFortran(m))) continue;
            double va = F0.cst, vb = 0.0;
            for (const auto& kv : F0.known) {
                const Affine& A = aff[kv.first.first];
                if (A.zero || A.a.empty()) continue;
                va += kv.second * (A.a[m] + (kv.first.second == 0 ? mParams.tau() * A.b[m] : 0.0));
                if (A.timed) vb += kv.second * A.b[m];
            }
            fa[m] = va;
            if (!fb.empty()) fb[m] = vb;
        }
    }

    // Border: every global-border node, at steps 1 and 2.  Four device
    // forms are tried at once: Dirichlet from one known field, the
    // StencilWidthOne mirror rule, a table of one linear rule per border
    // class (the set of faces the node lies on) -- the reference's Neumann
    // and Cauchy borders -- and one linear rule per border node (borders
    // whose coefficients change from node to node, such as the flux faces
    // of the tissue examples).
    int gfield = -1, gwhen = 0;
    bool dir_ok = true, mir_ok = true, tab_ok = true, nodes_ok = true;
    std::string tab_why, nodes_why;
    scafes_border_form forms[SCAFES_BORDER_CLASSES] = {};
    bool seen[SCAFES_BORDER_CLASSES] = {};
    int tab_g = -1;  // the one known field the table rules read as G
    std::vector<scafes_border_node_rule> node_rules;
    for (long long m = 0; m < mN; ++m) {
        const ScaFES_IntNtuple n = g.idxNodeScalar2TupleStyleFortran(m);
        if (!isBorder(n)) continue;
        gpu::Sym s1 = record<true>(n, 1, err)[0];
        if (!err.empty()) throw std::runtime_error("ScaFES::Problem: " + err);
        gpu::Sym s2 = record<true>(n, 2, err)[0];
        if (!err.empty()) throw std::runtime_error("ScaFES::Problem: " + err);
        if (s1.bad()) throw std::runtime_error("ScaFES::Problem: updateBorder is not linear: " + describe(s1));
        const auto& tt = s1.terms();
        // Dirichlet: u_new = K_j.
        const bool dir = tt.size() == 1 && tt[0].first.kind == 1 && tt[0].second == 1.0 && s1.constant() == 0.0 &&
                         same(s1, s2) && (gfield == -1 || (gfield == tt[0].first.a && gwhen == tt[0].first.b));
        if (dir && gfield == -1) { gfield = tt[0].first.a; gwhen = tt[0].first.b; }
        dir_ok = dir_ok && dir;
        // StencilWidthOne mirror: u_new = u + u(opposite) + s*2^(t-1).
        bool mirror = tt.size() == 2 && s1.constant() != 0.0 && s2.constant() == 2.0 * s1.constant() &&
                      std::fabs(s1.constant()) == 1.0;
        if (mirror)
            for (const auto& kv : tt)
                if (kv.first.kind != 0 || kv.second != 1.0) mirror = false;
        mir_ok = mir_ok && mirror;
        // The rule of this node alone.
        if (nodes_ok) {
            scafes_border_node_rule r = {};
            std::string why = nodeRule(s1, s2, aff, m, r);
            if (!why.empty()) {
                nodes_ok = false;
                nodes_why = why;
                node_rules.clear();
            } else {
                node_rules.push_back(r);
            }
        }
        if (tab_ok) {
            // Table rule of this node's class.
            int mask = 0;
            for (std::size_t p = 0; p < DIM; ++p) {
                if (n[p] == g.idxNodeFirst(p)) mask |= 1 << (2 * p);
                if (n[p] == g.idxNodeLast(p)) mask |= 1 << (2 * p + 1);
            }
            scafes_border_form r = {};
            std::string why = uniform ? tableRule(s1, s2, F0, aff, tab_g, r)
                                      : std::string("the inner update has variable coefficients");
            if (why.empty() && seen[mask] && std::memcmp(&r, &forms[mask], sizeof(r)) != 0)
                why = "the rule differs between nodes on the same faces";
            if (!why.empty()) {
                tab_ok = false;
                tab_why = why;
            } else {
                forms[mask] = r;
                seen[mask] = true;
            }
        }
        if (!dir_ok && !mir_ok && !tab_ok && !nodes_ok)
            throw std::runtime_error("ScaFES::Problem: updateBorder at node has no device form (" + tab_why + "; " +
                                     nodes_why + "): " + describe(s1));
    }
    int border = dir_ok ? SCAFES_BORDER_DIRICHLET
                 : mir_ok ? SCAFES_BORDER_MIRROR_POW2
                 : tab_ok ? SCAFES_BORDER_TABLE : SCAFES_BORDER_NODES;
    if (border == SCAFES_BORDER_TABLE) std::copy(forms, forms + SCAFES_BORDER_CLASSES, mForms);
    if (border == SCAFES_BORDER_NODES) mNodeRules.swap(node_rules);
    mWallClockTimes["record"] += std::chrono::duration<double>(clock::now() - t_rec).count();

    // 4. Device configuration.
    scafes_cfg cfg = {};
    cfg.dim = 3;
    for (int p = 0; p < 3; ++p) {
        cfg.n_nodes[p] = g.nNodes(p);
        cfg.coord_first[p] = g.coordNodeFirst()[p];
        cfg.coord_last[p] = g.coordNodeLast()[p];
    }
    cfg.tau = mParams.tau();
    cfg.t_start = mParams.timeIntervalStart();
    cfg.n_layers_at_border = mParams.nLayersAtBorder();
    cfg.precision = precisionCode();
    cfg.border = border;
    cfg.tile = mParams.gpuTile();
    const bool vc = !uniform || border == SCAFES_BORDER_NODES;
    if (!vc) {
        cfg.c0 = F0.c0;
        for (int p = 0; p < 3; ++p) cfg.cp[p] = F0.cp[p];
    } else {
        if (border == SCAFES_BORDER_MIRROR_POW2)
            throw std::runtime_error("ScaFES::Problem: variable coefficients with the mirror border have no device form");
        if (has_fb)
            throw std::runtime_error("ScaFES::Problem: variable coefficients take a source constant in time; "
                                     "a known field of the source changes with time");
        if (cfg.precision == SCAFES_PREC_F32X2)
            throw std::runtime_error("ScaFES::Problem: variable coefficients run with --gpuPrecision f64 or f32");
        // C0 = the node's centre weight, CA = its x-axis weight; the axis
        // factors cp[p] are the ratios of the axis weights, which must be
        // the same at every inner node (to rounding).
        const long long m0 = [&] {
            for (long long m = 0; m < mN; ++m)
                if (!isBorder(g.idxNodeScalar2TupleStyleFortran(m)) && cpn[0][m] != 0.0) return m;
            return -1LL;
        }();
        double kappa[3] = {1.0, 0.0, 0.0};
        if (m0 >= 0)
            for (int p = 1; p < 3; ++p) kappa[p] = cpn[p][m0] / cpn[0][m0];
        mC0.assign((std::size_t)mN, 0.0);
        mCA.assign((std::size_t)mN, 0.0);
        for (long long m = 0; m < mN; ++m) {
            if (isBorder(g.idxNodeScalar2TupleStyleFortran(m))) continue;
            const double ca = cpn[0][m];
            for (int p = 1; p < 3; ++p)
                if (std::fabs(ca * kappa[p] - cpn[p][m]) > 1e-13 * std::fabs(cpn[p][m]))
                    throw std::runtime_error("ScaFES::Problem: the axis weights of updateInner do not share one "
                                             "ratio over the nodes (anisotropic coefficients have no device form)");
            mC0[m] = c0n[m];
            mCA[m] = ca;
        }
        cfg.c0 = 0.0;
        for (int p = 0; p < 3; ++p) cfg.cp[p] = kappa[p];
    }
    cfg.cf = has_f ? 1.0 : 0.0;
    if (has_f) mFa.swap(fa);
    if (has_fb) mFb.swap(fb);
    if (border == SCAFES_BORDER_TABLE && tab_g >= 0) {
        const Affine& A = aff[tab_g];
        if (A.a.empty()) {
            fitTimePolynomial(tab_g);
        } else {
            mGa = A.a;
            if (A.timed) mGb = A.b;
        }
    }
    bool table_reads_f = false;
    if (border == SCAFES_BORDER_TABLE)
        for (int c = 0; c < SCAFES_BORDER_CLASSES; ++c) table_reads_f = table_reads_f || mForms[c].cf != 0.0;
    if (table_reads_f && !has_f)
        throw std::runtime_error("ScaFES::Problem: updateBorder reads a source the inner update does not have");
    if (border == SCAFES_BORDER_DIRICHLET && gfield >= 0 && !aff[gfield].zero) {
        const Affine& A = aff[gfield];
        if (A.a.empty())
            throw std::runtime_error("ScaFES::Problem: border field " + mNames[gfield] + " is not affine in time");
        mGa = A.a;
        if (gwhen == 1)
            for (long long m = 0; m < mN; ++m) mGa[m] -= mParams.tau() * A.b[m];
        if (A.timed) mGb = A.b;
    }
    mCfg = cfg;
    std::ostringstream os;
    if (vc)
        os << "star7-vc cp=(" << cfg.cp[0] << "," << cfg.cp[1] << "," << cfg.cp[2] << ")" << (uniform ? " uniform" : "");
    else
        os << "star7 c0=" << cfg.c0 << " cp=(" << cfg.cp[0] << "," << cfg.cp[1] << "," << cfg.cp[2] << ")";
    os << " source=" << (has_f ? (has_fb ? "affine" : "static") : "none")
       << " border=" << (border == SCAFES_BORDER_DIRICHLET ? "dirichlet"
                         : border == SCAFES_BORDER_MIRROR_POW2 ? "mirror"
                         : border == SCAFES_BORDER_TABLE ? "table" : "nodes");
    if (mGpoly) os << " G=quartic-in-time";
    if (border == SCAFES_BORDER_TABLE) {
        bool u4 = false;
        for (int c = 1; c < SCAFES_BORDER_CLASSES; ++c) u4 = u4 || mForms[c].cu4 != 0.0;
        if (u4) os << " u^4";
    }
    mSummary = os.str();
    mPrepared = true;
}

// A recorded form as a rule of the multi-field linear kernel, or why not.
template <class OWNPRBLM, typename CT, std::size_t DIM>
std::string Problem<OWNPRBLM, CT, DIM>::linearRule(const gpu::Sym& s, const std::vector<Affine>& aff,
                                                   std::vector<scafes_lin_term>& terms, double& cst) const {
    if (s.bad()) return "not linear in the unknowns: " + describe(s);
    terms.clear();
    cst = s.constant();
    for (const auto& kv : s.terms()) {
        const auto& k = kv.first;
        if (k.kind == 2) return "a power of an unknown: " + describe(s);
        if (k.kind == 1) {
            if (aff[k.a].zero) continue;  // a known field that is 0 everywhere
            return "a known field (" + mNames[k.a] + ") in a multi-field update: " + describe(s);
        }
        if (std::abs(k.b) > 1 || std::abs(k.c) > 1 || std::abs(k.d) > 1)
            return "a neighbour beyond one node: " + describe(s);
        terms.push_back(scafes_lin_term{k.a, k.b, k.c, k.d, kv.second});
    }
    if ((int)terms.size() > SCAFES_LIN_MAX_TERMS) return "more terms than the device rule holds: " + describe(s);
    return std::string();
}

template <class OWNPRBLM, typename CT, std::size_t DIM>
void Problem<OWNPRBLM, CT, DIM>::prepareLinear() {
    const std::size_t nu = mUnknownIdx.size();
    if (nu > SCAFES_LIN_MAX_FIELDS)
        throw std::runtime_error("ScaFES::Problem: more unknown fields than the multi-field kernel takes");
    if (mParams.nLayersAtBorder() != 1)
        throw std::runtime_error("ScaFES::Problem: the multi-field path takes one border layer");
    for (std::size_t u = 0; u < nu; ++u)
        if ((std::size_t)mUnknownIdx[u] < mWriteToFile.size() && mWriteToFile[mUnknownIdx[u]] != WriteHowOften::NEVER)
            throw std::runtime_error("ScaFES::Problem: field output is not available on the multi-field path");
    const Grid<DIM>& g = mGG.discreteDomain();
    const std::size_t nf = mNames.size();
    // Known fields at steps 0 and 1 (a multi-field update may only read
    // known fields that are 0 everywhere).
    evalKnownAt(0);
    std::vector<CT> k0 = mKnownNewStore;
    evalKnownAt(1);
    std::vector<CT> k1 = mKnownNewStore;
    std::vector<Affine> aff;
    fitAffine(aff, k0, k1);
    // Initial iterate of every unknown field (initInner/initBorder).
    std::copy(k0.begin(), k0.end(), mKnownNewStore.begin());
    mKnownOldStore = k0;
    {
        OWNPRBLM* self = static_cast<OWNPRBLM*>(this);
        for (auto& df : mVectUnknownDfsDomNew) df.time() = (CT)time(0);
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
        for (long long m = 0; m < mN; ++m) {
            const ScaFES_IntNtuple n = g.idxNodeScalar2TupleStyleFortran(m);
            if (isBorder(n)) self->template initBorder<CT>(mVectUnknownDfsDomNew, mVectParamsCurr, n, 0);
            else self->template initInner<CT>(mVectUnknownDfsDomNew, mVectParamsCurr, n, 0);
        }
    }
    std::copy(k1.begin(), k1.end(), mKnownNewStore.begin());
    (void)nf;
    mLinPhases = mUseLeapfrog ? 2 : 1;
    const std::size_t nrules = (std::size_t)mLinPhases * nu * SCAFES_BORDER_CLASSES;
    mLinTerms.assign(nrules, {});
    mLinCst.assign(nrules, 0.0);
    std::vector<bool> seen(nrules, false);
    std::string err;
    auto slot = [&](int ph, std::size_t f, int cls) { return ((std::size_t)ph * nu + f) * SCAFES_BORDER_CLASSES + cls; };
    auto take = [&](int ph, int cls, const std::vector<gpu::Sym>& out, const char* where) {
        for (std::size_t f = 0; f < nu; ++f) {
            std::vector<scafes_lin_term> terms;
            double cst = 0.0;
            const std::string why = linearRule(out[f], aff, terms, cst);
            if (!why.empty())
                throw std::runtime_error(std::string("ScaFES::Problem: ") + where + " of field " +
                                         mNames[mUnknownIdx[f]] + ": " + why);
            const std::size_t s = slot(ph, f, cls);
            if (!seen[s]) {
                mLinTerms[s] = terms;
                mLinCst[s] = cst;
                seen[s] = true;
                continue;
            }
            bool eq = cst == mLinCst[s] && terms.size() == mLinTerms[s].size();
            for (std::size_t k = 0; eq && k < terms.size(); ++k) {
                const auto& a = terms[k];
                bool found = false;
                for (const auto& b : mLinTerms[s])
                    if (a.src == b.src && a.dx == b.dx && a.dy == b.dy && a.dz == b.dz) { found = a.w == b.w; break; }
                eq = found;
            }
            if (!eq)
                throw std::runtime_error(std::string("ScaFES::Problem: ") + where + " of field " +
                                         mNames[mUnknownIdx[f]] +
                                         " differs between nodes of the same class or between time steps "
                                         "(variable coefficients have no multi-field device form)");
        }
    };
    auto cls_of = [&](const ScaFES_IntNtuple& n) {
        int mask = 0;
        for (std::size_t p = 0; p < DIM; ++p) {
            if (n[p] == g.idxNodeFirst(p)) mask |= 1 << (2 * p);
            if (n[p] == g.idxNodeLast(p)) mask |= 1 << (2 * p + 1);
        }
        return mask;
    };
    for (int ph = 0; ph < mLinPhases; ++ph) {
        for (long long m = 0; m < mN; ++m) {
            const ScaFES_IntNtuple n = g.idxNodeScalar2TupleStyleFortran(m);
            const bool border = isBorder(n);
            // Every border node; inner nodes on the lines through the first,
            // middle and last inner planes.
            if (!border) {
                int on = 0;
                for (std::size_t p = 0; p < DIM; ++p)
                    on += n[p] == 1 || n[p] == g.nNodes(p) / 2 || n[p] == g.nNodes(p) - 2;
                if (on + 1 < (int)DIM) continue;
            }
            for (int t = 1; t <= 2; ++t) {
                std::vector<gpu::Sym> out;
                if (ph == 0) out = border ? record<true, 1>(n, t, err) : record<false, 1>(n, t, err);
                else out = border ? record<true, 2>(n, t, err) : record<false, 2>(n, t, err);
                if (!err.empty()) throw std::runtime_error("ScaFES::Problem: " + err);
                take(ph, border ? cls_of(n) : 0, out,
                     ph == 0 ? (border ? "updateBorder" : "updateInner") : (border ? "updateBorder2" : "updateInner2"));
            }
        }
    }
    // Every other inner node at step 1 must give the inner rule too (a
    // coefficient read from a known field or a coordinate would not):
    // recorded in parallel and compared with the rules found above.
    auto equal_rule = [&](std::size_t s, const std::vector<scafes_lin_term>& terms, double cst) {
        if (cst != mLinCst[s] || terms.size() != mLinTerms[s].size()) return false;
        for (const auto& a : terms) {
            bool found = false;
            for (const auto& b : mLinTerms[s])
                if (a.src == b.src && a.dx == b.dx && a.dy == b.dy && a.dz == b.dz) { found = a.w == b.w; break; }
            if (!found) return false;
        }
        return true;
    };
    for (int ph = 0; ph < mLinPhases; ++ph) {
        long long bad = -1;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 4096)
#endif
        for (long long m = 0; m < mN; ++m) {
            long long seen_bad;
#ifdef _OPENMP
#pragma omp atomic read
#endif
            seen_bad = bad;
            if (seen_bad >= 0) continue;
            const ScaFES_IntNtuple n = g.idxNodeScalar2TupleStyleFortran(m);
            if (isBorder(n)) continue;
            std::string e2;
            const std::vector<gpu::Sym> out = ph == 0 ? record<false, 1>(n, 1, e2) : record<false, 2>(n, 1, e2);
            bool ok = e2.empty();
            for (std::size_t f = 0; ok && f < nu; ++f) {
                std::vector<scafes_lin_term> terms;
                double cst = 0.0;
                ok = linearRule(out[f], aff, terms, cst).empty() && equal_rule(slot(ph, f, 0), terms, cst);
            }
            if (!ok) {
#ifdef _OPENMP
#pragma omp critical(scafes_lin_bad)
#endif
                {
                    long long cur;
#ifdef _OPENMP
#pragma omp atomic read
#endif
                    cur = bad;
                    if (cur < 0 || m < cur) {
#ifdef _OPENMP
#pragma omp atomic write
#endif
                        bad = m;
                    }
                }
            }
        }
        if (bad >= 0) {
            const ScaFES_IntNtuple n = g.idxNodeScalar2TupleStyleFortran(bad);
            std::ostringstream e;
            e << "ScaFES::Problem: " << (ph == 0 ? "updateInner" : "updateInner2") << " at node (" << n[0] << ","
              << n[1] << "," << n[2] << ") differs from the other inner nodes' (coefficients that vary over the "
              << "nodes have no multi-field device form)";
            throw std::runtime_error(e.str());
        }
    }
    std::ostringstream os;
    os << "linear multi-field fields=" << nu << " phases=" << mLinPhases;
    mSummary = os.str();
    mLinear = true;
    mPrepared = true;
}

template <class OWNPRBLM, typename CT, std::size_t DIM>
void Problem<OWNPRBLM, CT, DIM>::runLinear() {
    const Grid<DIM>& g = mGG.discreteDomain();
    const std::size_t nu = mUnknownIdx.size();
    const int T = mParams.nTimesteps();
    int nn[3];
    for (int p = 0; p < 3; ++p) nn[p] = g.nNodes(p);
    scafes_lin* h = nullptr;
    if (scafes_lin_create(nn, (int)nu, mLinPhases, nullptr, &h) != SCAFES_OK)
        throw std::runtime_error(std::string("ScaFES::Problem (GPU): ") + scafes_last_error());
    auto lcheck = [&](int rc) {
        if (rc != SCAFES_OK) {
            const std::string msg = scafes_lin_last_error(h);
            scafes_lin_destroy(h);
            throw std::runtime_error("ScaFES::Problem (GPU): " + msg);
        }
    };
    for (int ph = 0; ph < mLinPhases; ++ph)
        for (std::size_t f = 0; f < nu; ++f)
            for (int c = 0; c < SCAFES_BORDER_CLASSES; ++c) {
                const std::size_t s = ((std::size_t)ph * nu + f) * SCAFES_BORDER_CLASSES + c;
                lcheck(scafes_lin_set_rule(h, ph + 1, (int)f, c, mLinTerms[s].data(), (int)mLinTerms[s].size(),
                                           mLinCst[s]));
            }
    std::vector<double> buf((std::size_t)mN);
    for (std::size_t u = 0; u < nu; ++u) {
        for (long long m = 0; m < mN; ++m) buf[m] = (double)mUnknownNewStore[u * mN + m];
        lcheck(scafes_lin_upload(h, (int)u, buf.data(), buf.size()));
    }
    lcheck(scafes_lin_step(h, T));
    float ms = 0.f;
    lcheck(scafes_lin_last_ms(h, &ms));
    mGpuMs = ms;
    for (std::size_t u = 0; u < nu; ++u) {
        lcheck(scafes_lin_download(h, (int)u, buf.data(), buf.size()));
        for (long long m = 0; m < mN; ++m) {
            mUnknownOldStore[u * mN + m] = (CT)buf[m];
            mUnknownNewStore[u * mN + m] = (CT)buf[m];
        }
    }
    scafes_lin_destroy(h);
    for (auto& df : mVectUnknownDfsDomOld) df.time() = (CT)time(T);
    for (auto& df : mVectUnknownDfsDomNew) df.time() = (CT)time(T);
}

template <class OWNPRBLM, typename CT, std::size_t DIM>
void Problem<OWNPRBLM, CT, DIM>::iterateOverTime() {
    using clock = std::chrono::steady_clock;
    auto t_all = clock::now();
    prepareDevice();
    if (mLinear) {
        runLinear();
        mWallClockTimes["iterate"] += std::chrono::duration<double>(clock::now() - t_all).count();
        if (mParams.outputLevel() > 0)
            std::cout << "ScaFES-GB300: " << mSummary << ", " << mParams.nTimesteps() << " steps in " << mGpuMs
                      << " ms" << std::endl;
        return;
    }
    const int T = mParams.nTimesteps();
    scafes_cfg cfg = mCfg;
    if (mHandle) { scafes_gpu_destroy(mHandle); mHandle = nullptr; }
    check(scafes_gpu_create(&cfg, &mHandle));
    if (cfg.border == SCAFES_BORDER_TABLE) check(scafes_gpu_set_border_forms(mHandle, mForms));
    if (cfg.border == SCAFES_BORDER_NODES)
        check(scafes_gpu_set_border_node_rules(mHandle, mNodeRules.data(), mNodeRules.size()));
    if (!mC0.empty()) {
        check(scafes_gpu_upload(mHandle, SCAFES_FIELD_C0, mC0.data(), mC0.size()));
        check(scafes_gpu_upload(mHandle, SCAFES_FIELD_CA, mCA.data(), mCA.size()));
    }
    if (!mFa.empty()) check(scafes_gpu_upload(mHandle, SCAFES_FIELD_F_A, mFa.data(), mFa.size()));
    if (!mFb.empty()) check(scafes_gpu_upload(mHandle, SCAFES_FIELD_F_B, mFb.data(), mFb.size()));
    if (!mGa.empty()) check(scafes_gpu_upload(mHandle, SCAFES_FIELD_G_A, mGa.data(), mGa.size()));
    if (!mGb.empty()) check(scafes_gpu_upload(mHandle, SCAFES_FIELD_G_B, mGb.data(), mGb.size()));
    if (mGpoly) {
        for (int k = 0; k < 3; ++k)
            check(scafes_gpu_upload(mHandle, SCAFES_FIELD_G_C + k, mGhi[k].data(), mGhi[k].size()));
        check(scafes_gpu_set_border_time_basis(mHandle, mGcenter, mGrate));
    }
    std::vector<double> u0(mUnknownNewStore.begin(), mUnknownNewStore.end());
    check(scafes_gpu_upload(mHandle, SCAFES_FIELD_U, u0.data(), u0.size()));
    int tile = cfg.tile;
    if (mParams.gpuAutotune()) check(scafes_gpu_autotune(mHandle, 5, &tile, nullptr));
    auto t_upd = clock::now();
    // Field output (writeDfsToFile, reference :4254-4340): the unknown field's
    // WriteHowOften maps to the snapshot writer, which copies and writes
    // while the sweeps run.
    const int uw = mUnknownIdx[0];
    const WriteHowOften how = (std::size_t)uw < mWriteToFile.size() ? mWriteToFile[uw] : WriteHowOften::NEVER;
    if (how == WriteHowOften::NEVER) {
        check(scafes_gpu_step(mHandle, T));
    } else {
        int interval = 0, flags = 0;
        switch (how) {
            case WriteHowOften::AT_START: flags = SCAFES_SNAP_START; break;
            case WriteHowOften::AT_END: flags = SCAFES_SNAP_END; break;
            case WriteHowOften::AT_START_AND_END: flags = SCAFES_SNAP_START | SCAFES_SNAP_END; break;
            case WriteHowOften::LIKE_GIVEN_AT_CL:
                interval = T;
                if (mParams.nSnapshots() > 0 && mParams.nSnapshots() <= T) interval = T / mParams.nSnapshots();
                flags = SCAFES_SNAP_START;
                break;
            default: interval = 1; flags = SCAFES_SNAP_START; break;  // ALWAYS
        }
        if (interval < 1) interval = 1;
        const std::string path = mParams.gpuSnapshotFile().empty() ? "scafes_" + mNames[uw] + ".snap"
                                                                   : mParams.gpuSnapshotFile();
        check(scafes_gpu_step_snapshots(mHandle, T, interval, flags, path.c_str()));
        mSnapshotFile = path;
    }
    std::vector<double> uT((std::size_t)mN);
    check(scafes_gpu_download(mHandle, SCAFES_FIELD_U, uT.data(), uT.size()));
    mWallClockTimes["update"] += std::chrono::duration<double>(clock::now() - t_upd).count();
    float ms = 0.f;
    if (T > 0) check(scafes_gpu_last_step_ms(mHandle, &ms));
    mGpuMs = ms;
    for (long long m = 0; m < mN; ++m) {
        mUnknownOldStore[m] = (CT)uT[m];
        mUnknownNewStore[m] = (CT)uT[m];
    }
    for (auto& df : mVectUnknownDfsDomOld) df.time() = (CT)time(T);
    for (auto& df : mVectUnknownDfsDomNew) df.time() = (CT)time(T);

    // Max-norm error against the exact solution at the final step.
    const int uf = mUnknownIdx[0];
    if (mComputeError[uf]) {
        auto t_err = clock::now();
        evalKnownAt(T);
        double e = 0.0;
        for (long long m = 0; m < mN; ++m)
            e = std::max(e, std::fabs((double)mUnknownOldStore[m] - (double)mKnownNewStore[uf * mN + m]));
        mErrLinf[uf] = e;
        mWallClockTimes["compErr"] += std::chrono::duration<double>(clock::now() - t_err).count();
        std::cout << "ScaFES-GB300: Local Linf error (" << mNames[uf] << ", t=" << time(T) << ") = " << e << std::endl;
    }
    mWallClockTimes["iterate"] += std::chrono::duration<double>(clock::now() - t_all).count();
    if (mParams.outputLevel() > 0) {
        std::cout << "ScaFES-GB300: " << mSummary << "\n";
        for (const auto& kv : mWallClockTimes)
            std::cout << "ScaFES-GB300:   t(" << kv.first << ") = " << kv.second << " s\n";
        std::cout << "ScaFES-GB300:   device sweeps: " << T << " steps in " << mGpuMs << " ms" << std::endl;
    }
}

}  // namespace ScaFES
#endif
