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
//  3. extract the update: updateInner<gpu::Sym> at probe nodes and
//     updateBorder<gpu::Sym> at every global-border node, at two time
//     steps, give linear forms that must match one of the device kernels --
//     the 7-point star with a source, and the Dirichlet or StencilWidthOne
//     mirror border -- otherwise the constructor-time contract is broken and
//     iterateOverTime throws (there is no CPU fallback);
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
        (void)nLayers; (void)defaultValue; (void)checkConvergence;
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
    template <bool BORDER>
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
        if (BORDER) self->template updateBorder<gpu::Sym>(vNew, vOld, n, t);
        else self->template updateInner<gpu::Sym>(vNew, vOld, n, t);
        err = rec.error;
        if (err.empty() && gpu::comparison_on_unknown())
            err = "update callback branches on the value of an unknown (not a linear stencil)";
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

    // What prepareDevice hands to the device run.
    bool mPrepared = false;
    scafes_cfg mCfg = {};
    std::vector<double> mFa, mFb, mGa, mGb;
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
    if (mUseLeapfrog)
        throw std::runtime_error("ScaFES::Problem: leapfrog problems are not mapped to a device kernel yet");
    if (mUnknownIdx.size() != 1)
        throw std::runtime_error("ScaFES::Problem: the device path takes exactly one unknown data field");
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
    gpu::Sym inner;
    bool first = true;
    for (int t = 1; t <= 2; ++t) {
        for (const auto& n : probes) {
            if (isBorder(n)) continue;
            gpu::Sym s = record<false>(n, t, err)[0];
            if (!err.empty()) throw std::runtime_error("ScaFES::Problem: " + err);
            if (first) { inner = s; first = false; }
            else if (!same(s, inner))
                throw std::runtime_error("ScaFES::Problem: updateInner differs between nodes or time steps "
                                         "(variable coefficients are not mapped to a device kernel): " +
                                         describe(inner) + " vs " + describe(s));
        }
    }
    if (first) throw std::runtime_error("ScaFES::Problem: the grid has no inner nodes");
    Form F = starForm(inner);

    // Border: every global-border node, at steps 1 and 2.  Three device
    // forms are tried at once: Dirichlet from one known field, the
    // StencilWidthOne mirror rule, and a table of one linear rule per border
    // class (the set of faces the node lies on) -- the reference's Neumann
    // and Cauchy borders.
    int gfield = -1, gwhen = 0;
    bool dir_ok = true, mir_ok = true, tab_ok = true;
    std::string tab_why;
    scafes_border_form forms[SCAFES_BORDER_CLASSES] = {};
    bool seen[SCAFES_BORDER_CLASSES] = {};
    int tab_g = -1;  // the one known field the table rules read as G
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
        if (!tab_ok) {
            if (!dir_ok && !mir_ok)
                throw std::runtime_error("ScaFES::Problem: updateBorder at node has no device form (" + tab_why +
                                         "): " + describe(s1));
            continue;
        }
        // Table rule of this node's class.
        int mask = 0;
        for (std::size_t p = 0; p < DIM; ++p) {
            if (n[p] == g.idxNodeFirst(p)) mask |= 1 << (2 * p);
            if (n[p] == g.idxNodeLast(p)) mask |= 1 << (2 * p + 1);
        }
        scafes_border_form r = {};
        std::string why = tableRule(s1, s2, F, aff, tab_g, r);
        if (why.empty() && seen[mask] && std::memcmp(&r, &forms[mask], sizeof(r)) != 0)
            why = "the rule differs between nodes on the same faces";
        if (!why.empty()) {
            tab_ok = false;
            tab_why = why;
            if (!dir_ok && !mir_ok)
                throw std::runtime_error("ScaFES::Problem: updateBorder at node has no device form (" + why + "): " +
                                         describe(s1));
            continue;
        }
        forms[mask] = r;
        seen[mask] = true;
    }
    int border = dir_ok ? SCAFES_BORDER_DIRICHLET : mir_ok ? SCAFES_BORDER_MIRROR_POW2 : SCAFES_BORDER_TABLE;
    if (border == SCAFES_BORDER_TABLE) std::copy(forms, forms + SCAFES_BORDER_CLASSES, mForms);
    mWallClockTimes["record"] += std::chrono::duration<double>(clock::now() - t_rec).count();

    // 4. Device run.
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
    cfg.c0 = F.c0;
    for (int p = 0; p < 3; ++p) cfg.cp[p] = F.cp[p];
    // Source: F(t_old) = cst + sum_j b_j K_j(t_old or t_new).
    std::vector<double> fa((std::size_t)mN, F.cst), fb;
    bool has_f = F.cst != 0.0, has_fb = false;
    for (const auto& kv : F.known) {
        const int j = kv.first.first;
        const bool is_new = kv.first.second == 0;
        const double bj = kv.second;
        const Affine& A = aff[j];
        if (A.zero) continue;
        if (A.a.empty())
            throw std::runtime_error("ScaFES::Problem: known field " + mNames[j] +
                                     " is not affine in time; the device path takes affine known fields");
        has_f = true;
        if (A.timed && fb.empty()) fb.assign((std::size_t)mN, 0.0);
        for (long long m = 0; m < mN; ++m) {
            fa[m] += bj * (A.a[m] + (is_new ? mParams.tau() * A.b[m] : 0.0));
            if (A.timed) fb[m] += bj * A.b[m];
        }
        has_fb = has_fb || A.timed;
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
    os << "star7 c0=" << cfg.c0 << " cp=(" << cfg.cp[0] << "," << cfg.cp[1] << "," << cfg.cp[2] << ")"
       << " source=" << (has_f ? (has_fb ? "affine" : "static") : "none")
       << " border=" << (border == SCAFES_BORDER_DIRICHLET ? "dirichlet"
                         : border == SCAFES_BORDER_MIRROR_POW2 ? "mirror" : "table");
    if (mGpoly) os << " G=quartic-in-time";
    if (border == SCAFES_BORDER_TABLE) {
        bool u4 = false;
        for (int c = 1; c < SCAFES_BORDER_CLASSES; ++c) u4 = u4 || mForms[c].cu4 != 0.0;
        if (u4) os << " u^4";
    }
    mSummary = os.str();
    mPrepared = true;
}

template <class OWNPRBLM, typename CT, std::size_t DIM>
void Problem<OWNPRBLM, CT, DIM>::iterateOverTime() {
    using clock = std::chrono::steady_clock;
    auto t_all = clock::now();
    prepareDevice();
    const int T = mParams.nTimesteps();
    scafes_cfg cfg = mCfg;
    if (mHandle) { scafes_gpu_destroy(mHandle); mHandle = nullptr; }
    check(scafes_gpu_create(&cfg, &mHandle));
    if (cfg.border == SCAFES_BORDER_TABLE) check(scafes_gpu_set_border_forms(mHandle, mForms));
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
