// ScaFES::Ntuple -- fixed-size tuple with component-wise operations, the
// index / coordinate type of the ScaFES callback interface
// (reference: src/ScaFES_Ntuple.hpp:86-686).
#ifndef SCAFES_GB300_NTUPLE_HPP
#define SCAFES_GB300_NTUPLE_HPP

#include <cstddef>
#include <ostream>
#include <vector>

namespace ScaFES {

template <typename TT, std::size_t NN>
class Ntuple {
public:
    Ntuple() { for (std::size_t i = 0; i < NN; ++i) v_[i] = TT(); }
    // Implicit, as in the reference: a scalar compares and combines with a
    // tuple component-wise.
    Ntuple(const TT& s) { for (std::size_t i = 0; i < NN; ++i) v_[i] = s; }
    Ntuple(const TT& a, const TT& b) {
        static_assert(NN == 2, "two components need NN == 2");
        v_[0] = a; v_[1] = b;
    }
    Ntuple(const TT& a, const TT& b, const TT& c) {
        static_assert(NN == 3, "three components need NN == 3");
        v_[0] = a; v_[1] = b; v_[2] = c;
    }
    explicit Ntuple(const std::vector<TT>& vec) {
        for (std::size_t i = 0; i < NN; ++i) v_[i] = i < vec.size() ? vec[i] : TT();
    }

    static constexpr std::size_t size() { return NN; }
    const TT& elem(const std::size_t& i) const { return v_[i]; }
    TT& elem(const std::size_t& i) { return v_[i]; }
    const TT& operator[](const std::size_t& i) const { return v_[i]; }
    TT& operator[](const std::size_t& i) { return v_[i]; }

    Ntuple& operator=(const TT& s) { for (std::size_t i = 0; i < NN; ++i) v_[i] = s; return *this; }
    Ntuple& operator+=(const Ntuple& r) { for (std::size_t i = 0; i < NN; ++i) v_[i] += r.v_[i]; return *this; }
    Ntuple& operator-=(const Ntuple& r) { for (std::size_t i = 0; i < NN; ++i) v_[i] -= r.v_[i]; return *this; }
    Ntuple& operator*=(const Ntuple& r) { for (std::size_t i = 0; i < NN; ++i) v_[i] *= r.v_[i]; return *this; }
    Ntuple& operator/=(const Ntuple& r) { for (std::size_t i = 0; i < NN; ++i) v_[i] /= r.v_[i]; return *this; }
    template <typename S> Ntuple& operator*=(const S& s) { for (std::size_t i = 0; i < NN; ++i) v_[i] *= s; return *this; }
    template <typename S> Ntuple& operator/=(const S& s) { for (std::size_t i = 0; i < NN; ++i) v_[i] /= s; return *this; }

    bool operator==(const Ntuple& r) const {
        for (std::size_t i = 0; i < NN; ++i) if (!(v_[i] == r.v_[i])) return false;
        return true;
    }
    bool operator!=(const Ntuple& r) const { return !(*this == r); }
    // Component-wise orderings, as in the reference: a < b iff a_i < b_i for all i.
    bool operator<(const Ntuple& r) const { for (std::size_t i = 0; i < NN; ++i) if (!(v_[i] < r.v_[i])) return false; return true; }
    bool operator<=(const Ntuple& r) const { for (std::size_t i = 0; i < NN; ++i) if (!(v_[i] <= r.v_[i])) return false; return true; }
    bool operator>(const Ntuple& r) const { for (std::size_t i = 0; i < NN; ++i) if (!(v_[i] > r.v_[i])) return false; return true; }
    bool operator>=(const Ntuple& r) const { for (std::size_t i = 0; i < NN; ++i) if (!(v_[i] >= r.v_[i])) return false; return true; }

    TT sum() const { TT s = TT(); for (std::size_t i = 0; i < NN; ++i) s += v_[i]; return s; }
    TT prod() const { TT s = TT(1); for (std::size_t i = 0; i < NN; ++i) s *= v_[i]; return s; }

private:
    TT v_[NN];
};

template <typename TT, std::size_t NN>
Ntuple<TT, NN> operator+(Ntuple<TT, NN> a, const Ntuple<TT, NN>& b) { return a += b; }
template <typename TT, std::size_t NN>
Ntuple<TT, NN> operator-(Ntuple<TT, NN> a, const Ntuple<TT, NN>& b) { return a -= b; }
template <typename TT, std::size_t NN>
Ntuple<TT, NN> operator*(Ntuple<TT, NN> a, const Ntuple<TT, NN>& b) { return a *= b; }
template <typename TT, std::size_t NN>
Ntuple<TT, NN> operator-(Ntuple<TT, NN> a) { for (std::size_t i = 0; i < NN; ++i) a[i] = -a[i]; return a; }

template <typename TT, std::size_t NN>
std::ostream& operator<<(std::ostream& os, const Ntuple<TT, NN>& t) {
    os << "(";
    for (std::size_t i = 0; i < NN; ++i) os << (i ? ", " : "") << t[i];
    return os << ")";
}

}  // namespace ScaFES
#endif
