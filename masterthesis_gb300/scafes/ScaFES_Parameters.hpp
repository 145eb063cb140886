// ScaFES::Parameters -- run configuration of a problem.
//
// Accepts the reference's command-line options (src/ScaFES_Parameters.hpp:
// 474-540; "--name=value" or "--name value"; tuples as "8x8x8") without
// Boost, plus explicit setters.  Options the GPU path has no use for
// (partitioning, files, ADOL-C, MPI modes) are accepted and ignored.
// GPU-specific options:
//   --gpuPrecision=f64|f32x2|f32   arithmetic of the unknown field (f64)
//   --gpuTile=0..4                 sweep tile variant, 0 = default
//   --gpuAutotune=0|1              time the tile variants before running
//   --gpuSnapshotFile=PATH         where fields with writeToFile != NEVER
//                                  are written (default scafes_<field>.snap)
#ifndef SCAFES_GB300_PARAMETERS_HPP
#define SCAFES_GB300_PARAMETERS_HPP

#include <cstdlib>
#include <iostream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace ScaFES {

class Parameters {
public:
    Parameters(int argc = 0, char* argv[] = nullptr)
        : mDim(3), mNnodes(3, 32), mCoordNodeFirst(3, 0.0), mCoordNodeLast(3, 1.0) {
        bool have_tau = false, have_end = false, have_n = false;
        for (int i = 1; i < argc; ++i) {
            std::string a = argv[i];
            if (a.size() < 3 || a.compare(0, 2, "--") != 0) continue;
            std::string key = a.substr(2), val;
            const std::size_t eq = key.find('=');
            if (eq != std::string::npos) {
                val = key.substr(eq + 1);
                key = key.substr(0, eq);
            } else if (i + 1 < argc && std::string(argv[i + 1]).compare(0, 2, "--") != 0) {
                val = argv[++i];
            }
            if (key == "dim") mDim = std::atoi(val.c_str());
            else if (key == "nNodes") mNnodes = tuple<int>(val);
            else if (key == "coordNodeFirst") mCoordNodeFirst = tuple<double>(val);
            else if (key == "coordNodeLast") mCoordNodeLast = tuple<double>(val);
            else if (key == "nTimesteps") { mNtimesteps = std::atoi(val.c_str()); have_n = true; }
            else if (key == "tau") { mTau = std::atof(val.c_str()); have_tau = true; }
            else if (key == "starttime") mTimeIntervalStart = std::atof(val.c_str());
            else if (key == "endtime") { mTimeIntervalEnd = std::atof(val.c_str()); have_end = true; }
            else if (key == "nLayersAtBorder") mNlayersAtBorder = std::atoi(val.c_str());
            else if (key == "outputlevel") mOutputLevel = std::atoi(val.c_str());
            else if (key == "gpuPrecision") mGpuPrecision = val;
            else if (key == "gpuTile") mGpuTile = std::atoi(val.c_str());
            else if (key == "gpuAutotune") mGpuAutotune = std::atoi(val.c_str()) != 0;
            else if (key == "nSnapshots") mNsnapshots = std::atoi(val.c_str());
            else if (key == "gpuSnapshotFile") mGpuSnapshotFile = val;
            else if (key == "initfile") { mNameInitFile = val; mReadInitFile = true; }
            else if (key == "initfileIndex") mInitFileIndex = std::atoi(val.c_str());
        }
        mNnodes.resize(mDim, mNnodes.empty() ? 32 : mNnodes.back());
        mCoordNodeFirst.resize(mDim, 0.0);
        mCoordNodeLast.resize(mDim, 1.0);
        // Time step width as in the reference (src/ScaFES_Parameters.hpp:769-795).
        if (!have_tau) {
            if (have_end && have_n) mTau = mNtimesteps == 0 ? 0.0 : (mTimeIntervalEnd - mTimeIntervalStart) / mNtimesteps;
            else mTau = (mTimeIntervalEnd - mTimeIntervalStart) / (mNtimesteps > 0 ? mNtimesteps : 1);
        }
    }

    const int& dim() const { return mDim; }
    const std::vector<int>& nNodes() const { return mNnodes; }
    const std::vector<double>& coordNodeFirst() const { return mCoordNodeFirst; }
    const std::vector<double>& coordNodeLast() const { return mCoordNodeLast; }
    const double& timeIntervalStart() const { return mTimeIntervalStart; }
    const double& timeIntervalEnd() const { return mTimeIntervalEnd; }
    const int& nTimesteps() const { return mNtimesteps; }
    const double& tau() const { return mTau; }
    const int& nLayersAtBorder() const { return mNlayersAtBorder; }
    const int& outputLevel() const { return mOutputLevel; }
    const std::string& gpuPrecision() const { return mGpuPrecision; }
    const int& gpuTile() const { return mGpuTile; }
    bool gpuAutotune() const { return mGpuAutotune; }
    const int& nSnapshots() const { return mNsnapshots; }
    const std::string& gpuSnapshotFile() const { return mGpuSnapshotFile; }
    // The reference's single-rank answers.
    int rank() const { return 0; }
    int rankOutput() const { return 0; }
    bool enabledAdolc() const { return false; }
    // --initfile (src/ScaFES_Parameters.hpp:518, 937-941): the unknown
    // fields start from a file instead of initInner/initBorder.  Here the
    // file is a snapshot file of the GPU path (scafes_gpu_step_snapshots);
    // --initfileIndex picks the snapshot (default 0, the reference's
    // readDfsFromFile(0); -1 = the last one).
    const bool& readInitFile() const { return mReadInitFile; }
    const std::string& nameInitFile() const { return mNameInitFile; }
    const int& initFileIndex() const { return mInitFileIndex; }

    void setDim(int d) { mDim = d; mNnodes.resize(d, 32); mCoordNodeFirst.resize(d, 0.0); mCoordNodeLast.resize(d, 1.0); }
    void setNnodes(const std::vector<int>& n) { mNnodes = n; }
    void setCoordNodeFirst(const std::vector<double>& c) { mCoordNodeFirst = c; }
    void setCoordNodeLast(const std::vector<double>& c) { mCoordNodeLast = c; }
    void setTimeInterval(double t0, double t1) { mTimeIntervalStart = t0; mTimeIntervalEnd = t1; }
    void setNtimesteps(int n) { mNtimesteps = n; }
    void setTau(double tau) { mTau = tau; }
    void setNlayersAtBorder(int n) { mNlayersAtBorder = n; }
    void setOutputLevel(int l) { mOutputLevel = l; }
    void setGpuPrecision(const std::string& p) { mGpuPrecision = p; }
    void setGpuTile(int t) { mGpuTile = t; }
    void setGpuAutotune(bool a) { mGpuAutotune = a; }
    void setNsnapshots(int n) { mNsnapshots = n; }
    void setGpuSnapshotFile(const std::string& f) { mGpuSnapshotFile = f; }
    void setInitFile(const std::string& f, int index = 0) {
        mNameInitFile = f;
        mReadInitFile = !f.empty();
        mInitFileIndex = index;
    }

private:
    template <typename T>
    static std::vector<T> tuple(const std::string& s) {
        std::vector<T> out;
        std::stringstream ss(s);
        std::string item;
        while (std::getline(ss, item, 'x')) {
            std::stringstream is(item);
            T v{};
            is >> v;
            out.push_back(v);
        }
        return out;
    }

    int mDim;
    std::vector<int> mNnodes;
    std::vector<double> mCoordNodeFirst, mCoordNodeLast;
    double mTimeIntervalStart = 0.0, mTimeIntervalEnd = 1.0;
    int mNtimesteps = 1;
    double mTau = 1.0;
    int mNlayersAtBorder = 1;
    int mOutputLevel = 0;
    std::string mGpuPrecision = "f64";
    int mGpuTile = 0;
    bool mGpuAutotune = false;
    int mNsnapshots = 1;  // the reference's default (src/ScaFES_Parameters.hpp:446)
    std::string mGpuSnapshotFile;
    std::string mNameInitFile = "EMPTYINITFILE";  // the reference's default name (:451)
    bool mReadInitFile = false;
    int mInitFileIndex = 0;
};

}  // namespace ScaFES
#endif
