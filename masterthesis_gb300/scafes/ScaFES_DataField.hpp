// ScaFES::DataField -- a field on the global grid as the callbacks see it.
//
// DataField<CT, DIM> with an arithmetic CT is a view of host storage owned
// by the Problem (nodes in Fortran order, x fastest, plus the time of the
// iterate).  The reference's DataField (src/ScaFES_DataField.hpp:99-586)
// also carries the MPI ghost layer and halo buffers; here the device holds
// the grid and the border pass replaces the ghost exchange, so the host view
// needs neither.
//
// DataField<gpu::Sym, DIM> is the recording view used to extract a stencil:
// reading field f at node n yields the symbol U_f(n - centre); the output
// view exposes one slot per field at the centre node.
#ifndef SCAFES_GB300_DATAFIELD_HPP
#define SCAFES_GB300_DATAFIELD_HPP

#include <deque>
#include <stdexcept>
#include <string>
#include <vector>

#include "ScaFES_Grid.hpp"
#include "ScaFES_Sym.hpp"

namespace ScaFES {

// How often a field is written to file (reference: src/ScaFES_DataFile.hpp:
// 24-32).  The GPU path writes no files; the values are accepted.
enum class WriteHowOften { NEVER = 1, AT_START = 2, AT_END = 3, AT_START_AND_END = 4, LIKE_GIVEN_AT_CL = 8, ALWAYS = 16 };

template <typename CT, std::size_t DIM>
class DataField {
public:
    DataField() = default;
    DataField(const std::string& name, const GridGlobal<DIM>* gg, CT* data, int stencilWidth)
        : mName(name), mGG(gg), mData(data), mStencilWidth(stencilWidth) {}

    CT& operator()(const Ntuple<int, DIM>& n) const {
        const Grid<DIM>& g = mGG->discreteDomain();
        if (!g.inside(n)) {
            // The reference reads outside its memory here (a connect()
            // sentinel); a zero stands in so host-side evaluation stays defined.
            mOutside = CT();
            return mOutside;
        }
        return mData[g.idxNodeTuple2ScalarStyleFortran(n)];
    }
    CT& operator()(const unsigned long& memoryPos) const { return mData[memoryPos]; }
    CT& time() const { return mTime; }
    const std::string& name() const { return mName; }
    const int& stencilWidth() const { return mStencilWidth; }
    const GridGlobal<DIM>& gridGlobal() const { return *mGG; }
    CT* data() const { return mData; }
    void setData(CT* d) { mData = d; }

private:
    std::string mName;
    const GridGlobal<DIM>* mGG = nullptr;
    CT* mData = nullptr;
    int mStencilWidth = 0;
    mutable CT mTime = CT();
    mutable CT mOutside = CT();
};

namespace gpu {

// Shared state of one recording: the centre node, the output slots and the
// symbols handed out for reads.
template <std::size_t DIM>
struct Recorder {
    Ntuple<int, DIM> centre;
    std::vector<Sym> out;           // one slot per unknown field
    std::deque<Sym> reads;          // stable storage for read results
    std::string error;
    const Grid<DIM>* grid = nullptr;
};

}  // namespace gpu

template <std::size_t DIM>
class DataField<gpu::Sym, DIM> {
public:
    DataField() = default;
    DataField(const std::string& name, const GridGlobal<DIM>* gg, gpu::Recorder<DIM>* rec, int field,
              bool is_output, int stencilWidth)
        : mName(name), mGG(gg), mRec(rec), mField(field), mOutput(is_output), mStencilWidth(stencilWidth) {}

    gpu::Sym& operator()(const Ntuple<int, DIM>& n) const {
        if (mOutput) {
            if (n != mRec->centre && mRec->error.empty())
                mRec->error = "update callback accesses the new iterate away from its own node";
            return mRec->out[mField];
        }
        if (!mGG->discreteDomain().inside(n)) {
            if (mRec->error.empty()) mRec->error = "update callback reads a node outside the domain";
            mRec->reads.push_back(gpu::Sym::nonlinear());
            return mRec->reads.back();
        }
        int d[3] = {0, 0, 0};
        for (std::size_t p = 0; p < DIM; ++p) d[p] = n[p] - mRec->centre[p];
        mRec->reads.push_back(gpu::Sym::unknown(mField, d[0], d[1], d[2]));
        return mRec->reads.back();
    }
    gpu::Sym& time() const { return mTime; }
    const std::string& name() const { return mName; }
    const int& stencilWidth() const { return mStencilWidth; }
    const GridGlobal<DIM>& gridGlobal() const { return *mGG; }

private:
    std::string mName;
    const GridGlobal<DIM>* mGG = nullptr;
    gpu::Recorder<DIM>* mRec = nullptr;
    int mField = 0;
    bool mOutput = false;
    int mStencilWidth = 0;
    mutable gpu::Sym mTime;
};

}  // namespace ScaFES
#endif
