// ScaFES::Grid and ScaFES::GridGlobal -- the discrete domain of a problem.
//
// Index semantics as in the reference: grid sizes h_p =
// (last_p - first_p)/(n_p - 1) (src/ScaFES_Grid.hpp:551-553), coordinates
// first_p + h_p*(i_p - i0_p) (:721-733), neighbour in direction dir with a
// negative sentinel tuple -(dir+1) at the domain edge (:887-921), and
// Fortran node order (x fastest, :956-968).  One GPU owns the whole domain,
// so GridGlobal has a single partition equal to the discrete domain.
#ifndef SCAFES_GB300_GRID_HPP
#define SCAFES_GB300_GRID_HPP

#include <stdexcept>

#include "ScaFES_Ntuple.hpp"
#include "ScaFES_Parameters.hpp"

namespace ScaFES {

template <std::size_t DIM>
class Grid {
public:
    Grid() = default;
    Grid(const Ntuple<int, DIM>& first, const Ntuple<int, DIM>& last,
         const Ntuple<double, DIM>& coordFirst, const Ntuple<double, DIM>& coordLast)
        : mFirst(first), mLast(last), mN(last - first + Ntuple<int, DIM>(1)),
          mCoordFirst(coordFirst), mCoordLast(coordLast) {
        for (std::size_t p = 0; p < DIM; ++p)
            mH[p] = mN[p] > 1 ? (coordLast[p] - coordFirst[p]) / (mN[p] - 1) : 0.0;
    }

    const Ntuple<int, DIM>& idxNodeFirst() const { return mFirst; }
    const Ntuple<int, DIM>& idxNodeLast() const { return mLast; }
    const int& idxNodeFirst(const int& p) const { return mFirst[p]; }
    const int& idxNodeLast(const int& p) const { return mLast[p]; }
    const Ntuple<int, DIM>& nNodes() const { return mN; }
    const int& nNodes(const int& p) const { return mN[p]; }
    const Ntuple<double, DIM>& coordNodeFirst() const { return mCoordFirst; }
    const Ntuple<double, DIM>& coordNodeLast() const { return mCoordLast; }
    const double& gridsize(const int& p) const { return mH[p]; }
    const Ntuple<double, DIM>& gridsize() const { return mH; }
    long long nNodesTotal() const { long long s = 1; for (std::size_t p = 0; p < DIM; ++p) s *= mN[p]; return s; }

    Ntuple<double, DIM> coordinates(const Ntuple<int, DIM>& n) const {
        Ntuple<double, DIM> c(0.0);
        for (std::size_t p = 0; p < DIM; ++p) c[p] = mCoordFirst[p] + mH[p] * (n[p] - mFirst[p]);
        return c;
    }

    Ntuple<int, DIM> neigh(const Ntuple<int, DIM>& n, const int& dir) const {
        Ntuple<int, DIM> r(n);
        const int p = dir / 2;
        const bool edge = (dir % 2 == 0) ? n[p] == mFirst[p] : n[p] == mLast[p];
        if (edge) return Ntuple<int, DIM>(-(dir + 1));
        r[p] += (dir % 2 == 0) ? -1 : 1;
        return r;
    }

    bool inside(const Ntuple<int, DIM>& n) const {
        for (std::size_t p = 0; p < DIM; ++p) if (n[p] < mFirst[p] || n[p] > mLast[p]) return false;
        return true;
    }

    // Fortran order: x fastest.
    long long idxNodeTuple2ScalarStyleFortran(const Ntuple<int, DIM>& n) const {
        long long s = n[DIM - 1] - mFirst[DIM - 1];
        for (int p = (int)DIM - 2; p >= 0; --p) s = s * mN[p] + (n[p] - mFirst[p]);
        return s;
    }
    Ntuple<int, DIM> idxNodeScalar2TupleStyleFortran(long long s) const {
        Ntuple<int, DIM> n;
        for (std::size_t p = 0; p < DIM; ++p) { n[p] = (int)(s % mN[p]) + mFirst[p]; s /= mN[p]; }
        return n;
    }

private:
    Ntuple<int, DIM> mFirst, mLast, mN;
    Ntuple<double, DIM> mCoordFirst, mCoordLast, mH;
};

template <std::size_t DIM>
class GridGlobal {
public:
    // Node-kind bits (reference: src/ScaFES_GridGlobal.hpp:140-150).
    static const short SCAFES_GLOBAL_INNER_NODE = 4;
    static const short SCAFES_GLOBAL_BORDER_NODE = 8;
    static const short SCAFES_PARTITION_INNER_NODE = 128;
    static const short SCAFES_PARTITION_BORDER_NODE = 256;

    explicit GridGlobal(const Parameters& params) {
        if ((int)DIM != params.dim())
            throw std::runtime_error("ScaFES::GridGlobal: DIM differs from the --dim parameter");
        Ntuple<int, DIM> first(0), last(0);
        Ntuple<double, DIM> cf(0.0), cl(0.0);
        for (std::size_t p = 0; p < DIM; ++p) {
            if (params.nNodes()[p] < 2) throw std::runtime_error("ScaFES::GridGlobal: fewer than 2 nodes in a direction");
            last[p] = params.nNodes()[p] - 1;
            cf[p] = params.coordNodeFirst()[p];
            cl[p] = params.coordNodeLast()[p];
        }
        mDomain = Grid<DIM>(first, last, cf, cl);
    }
    const Grid<DIM>& discreteDomain() const { return mDomain; }
    const Grid<DIM>& partition(int) const { return mDomain; }
    int nPartitions() const { return 1; }

private:
    Grid<DIM> mDomain;
};

}  // namespace ScaFES
#endif
