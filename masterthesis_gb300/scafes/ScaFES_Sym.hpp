// Recording scalar used to extract the stencil of a user's update callback.
//
// ScaFES makes every per-node callback a template on its scalar type TT
// (src/ScaFES_Problem.hpp:433-449), which is how the reference substitutes
// ADOL-C's adouble (:5646-5652).  The drop-in Problem uses the same hook:
// it instantiates updateInner<Sym> / updateBorder<Sym>, where reading
// vOld[f](n) yields the symbol "unknown field f at offset n - centre", and
// the arithmetic of the callback builds a form
//     sum_k a_k * U_{f_k}(centre + d_k) + sum_j b_j * K_j(t or t-1) + c
//     + sum_{p=2..4} e_p * U_f(centre)^p.
// The powers of the node's own unknown come from products of forms that
// hold nothing but that unknown (the u^4 radiative flux of
// tests/system/PennesBioheatEqnFDM/Radiation/Radiation.hpp:146-159).  Any
// other product of two non-constant forms, a power above 4, or a
// non-constant argument to pow/exp/... marks the form as non-linear; such a
// callback cannot be mapped to a stencil kernel and the Problem refuses it
// with an error (there is no CPU fallback).
//
// Known fields enter through ScaFES::gpu::Known, the value returned by
// knownDf/knownDfNew/knownDfOld: it carries both the numeric value (so the
// same expression still works with TT = double) and its symbol.
#ifndef SCAFES_GB300_SYM_HPP
#define SCAFES_GB300_SYM_HPP

#include <cmath>
#include <type_traits>
#include <utility>
#include <vector>

namespace ScaFES {
namespace gpu {

// Set when a callback converts a form that holds unknowns to a number (a
// branch or an elementary function on the value of an unknown, or an
// assignment of such a form to a CT variable): such a callback is not a
// linear stencil, and the Problem refuses it.
inline bool& converted_unknown() {
    static thread_local bool flag = false;
    return flag;
}

// A term key: kind 0 = unknown field `a` at offset (b, c, d);
//             kind 1 = known field `a` at time level `b` (0 new, 1 old);
//             kind 2 = unknown field `a` at the centre node, to the power b.
struct TermKey {
    int kind, a, b, c, d;
    bool operator==(const TermKey& o) const {
        return kind == o.kind && a == o.a && b == o.b && c == o.c && d == o.d;
    }
};

class Sym {
public:
    Sym() = default;
    template <class A, class = typename std::enable_if<std::is_arithmetic<A>::value>::type>
    Sym(A v) : c_(static_cast<double>(v)) {}

    static Sym unknown(int field, int dx, int dy, int dz) {
        Sym s;
        s.t_.push_back({{0, field, dx, dy, dz}, 1.0});
        return s;
    }
    static Sym known(int idx, int when) {
        Sym s;
        s.t_.push_back({{1, idx, when, 0, 0}, 1.0});
        return s;
    }
    static Sym nonlinear() {
        Sym s;
        s.bad_ = true;
        return s;
    }

    bool is_const() const { return t_.empty() && !bad_; }
    // The number a form stands for: its constant, when it holds no unknown.
    // Converting a form with unknowns yields its constant part and marks the
    // recording as not a stencil (converted_unknown).
    operator double() const {
        if (!is_const()) converted_unknown() = true;
        return c_;
    }
    bool bad() const { return bad_; }
    double constant() const { return c_; }
    const std::vector<std::pair<TermKey, double>>& terms() const { return t_; }

    Sym& operator+=(const Sym& o) {
        c_ += o.c_;
        bad_ = bad_ || o.bad_;
        for (const auto& kv : o.t_) add(kv.first, kv.second);
        return *this;
    }
    Sym& operator-=(const Sym& o) {
        c_ -= o.c_;
        bad_ = bad_ || o.bad_;
        for (const auto& kv : o.t_) add(kv.first, -kv.second);
        return *this;
    }
    Sym& operator*=(const Sym& o) {
        if (o.is_const()) {
            scale(o.c_);
        } else if (is_const()) {
            const double k = c_;
            *this = o;
            scale(k);
        } else {
            *this = centre_product(*this, o);
        }
        return *this;
    }
    Sym& operator/=(const Sym& o) {
        if (o.is_const()) {
            c_ /= o.c_;
            for (auto& kv : t_) kv.second /= o.c_;
        } else {
            bad_ = true;
        }
        return *this;
    }
    Sym operator-() const {
        Sym s(*this);
        s.scale(-1.0);
        return s;
    }
    Sym operator+() const { return *this; }

private:
    // Coefficients 0..4 of a form that is a polynomial in the centre unknown
    // of one field; false for anything else.
    static bool centre_poly(const Sym& s, int& field, double co[5]) {
        if (s.bad_) return false;
        field = -1;
        for (int p = 0; p < 5; ++p) co[p] = 0.0;
        co[0] = s.c_;
        for (const auto& kv : s.t_) {
            const TermKey& k = kv.first;
            int power;
            if (k.kind == 0 && k.b == 0 && k.c == 0 && k.d == 0) power = 1;
            else if (k.kind == 2) power = k.b;
            else return false;
            if (field != -1 && k.a != field) return false;
            field = k.a;
            co[power] += kv.second;
        }
        return true;
    }
    static Sym centre_product(const Sym& a, const Sym& b) {
        int fa, fb;
        double ca[5], cb[5], cr[9] = {};
        if (!centre_poly(a, fa, ca) || !centre_poly(b, fb, cb) || fa != fb) return nonlinear();
        for (int i = 0; i < 5; ++i)
            for (int j = 0; j < 5; ++j) cr[i + j] += ca[i] * cb[j];
        for (int p = 5; p < 9; ++p)
            if (cr[p] != 0.0) return nonlinear();
        Sym r(cr[0]);
        if (cr[1] != 0.0) r.t_.push_back({{0, fa, 0, 0, 0}, cr[1]});
        for (int p = 2; p < 5; ++p)
            if (cr[p] != 0.0) r.t_.push_back({{2, fa, p, 0, 0}, cr[p]});
        return r;
    }

    void add(const TermKey& k, double v) {
        for (auto& kv : t_) {
            if (kv.first == k) {
                kv.second += v;
                return;
            }
        }
        t_.push_back({k, v});
    }
    void scale(double k) {
        c_ *= k;
        for (auto& kv : t_) kv.second *= k;
    }

    std::vector<std::pair<TermKey, double>> t_;
    double c_ = 0.0;
    bool bad_ = false;
};

inline Sym operator+(Sym a, const Sym& b) { return a += b; }
inline Sym operator-(Sym a, const Sym& b) { return a -= b; }
inline Sym operator*(Sym a, const Sym& b) { return a *= b; }
inline Sym operator/(Sym a, const Sym& b) { return a /= b; }
// Mixed forms with a number: exact matches, so that the built-in double
// operators (reachable through Sym's conversion) never compete.
inline Sym operator+(Sym a, double b) { return a += Sym(b); }
inline Sym operator+(double a, const Sym& b) { return Sym(a) += b; }
inline Sym operator-(Sym a, double b) { return a -= Sym(b); }
inline Sym operator-(double a, const Sym& b) { return Sym(a) -= b; }
inline Sym operator*(Sym a, double b) { return a *= Sym(b); }
inline Sym operator*(double a, const Sym& b) { return Sym(a) *= b; }
inline Sym operator/(Sym a, double b) { return a /= Sym(b); }
inline Sym operator/(double a, const Sym& b) { return Sym(a) /= b; }

// Comparisons are only meaningful between constants.  A branch on the value
// of an unknown is not a stencil: it sets a per-thread flag that the
// recording checks, and the Problem refuses the callback.
inline bool& comparison_on_unknown() {
    static thread_local bool flag = false;
    return flag;
}
#define SCAFES_SYM_CMP(OP)                                                    \
    inline bool operator OP(const Sym& a, const Sym& b) {                     \
        if (!a.is_const() || !b.is_const()) {                                 \
            comparison_on_unknown() = true;                                   \
            return false;                                                     \
        }                                                                     \
        return a.constant() OP b.constant();                                  \
    }                                                                         \
    inline bool operator OP(const Sym& a, double b) { return a OP Sym(b); }   \
    inline bool operator OP(double a, const Sym& b) { return Sym(a) OP b; }
SCAFES_SYM_CMP(<)
SCAFES_SYM_CMP(<=)
SCAFES_SYM_CMP(>)
SCAFES_SYM_CMP(>=)
SCAFES_SYM_CMP(==)
SCAFES_SYM_CMP(!=)
#undef SCAFES_SYM_CMP

// Elementary functions: fine on constants, non-linear otherwise.
#define SCAFES_SYM_UNARY(FN)                                           \
    inline Sym FN(const Sym& a) {                                      \
        return a.is_const() ? Sym(std::FN(a.constant())) : Sym::nonlinear(); \
    }
SCAFES_SYM_UNARY(sqrt)
SCAFES_SYM_UNARY(exp)
SCAFES_SYM_UNARY(log)
SCAFES_SYM_UNARY(sin)
SCAFES_SYM_UNARY(cos)
SCAFES_SYM_UNARY(tan)
SCAFES_SYM_UNARY(fabs)
#undef SCAFES_SYM_UNARY
inline Sym abs(const Sym& a) { return fabs(a); }
inline Sym pow(const Sym& a, const Sym& b);
inline Sym pow(const Sym& a, double b) { return pow(a, Sym(b)); }
inline Sym pow(const Sym& a, int b) { return pow(a, Sym(b)); }
inline Sym pow(const Sym& a, const Sym& b) {
    if (a.is_const() && b.is_const()) return Sym(std::pow(a.constant(), b.constant()));
    if (b.is_const() && b.constant() == 1.0) return a;
    if (b.is_const() && (b.constant() == 2.0 || b.constant() == 3.0 || b.constant() == 4.0)) {
        Sym r = a;
        for (int p = 1; p < (int)b.constant(); ++p) r *= a;  // non-linear unless a is the centre unknown
        return r;
    }
    return Sym::nonlinear();
}

// Value + symbol of a known-field read (see the header comment).
class Known {
public:
    Known(double v, Sym s) : v_(v), s_(std::move(s)) {}
    operator double() const { return v_; }
    operator Sym() const { return s_; }
    double value() const { return v_; }
    const Sym& sym() const { return s_; }

    Known operator-() const { return Known(-v_, -s_); }
    friend Known operator+(const Known& a, const Known& b) { return Known(a.v_ + b.v_, a.s_ + b.s_); }
    friend Known operator-(const Known& a, const Known& b) { return Known(a.v_ - b.v_, a.s_ - b.s_); }
    friend Known operator*(const Known& a, const Known& b) { return Known(a.v_ * b.v_, a.s_ * b.s_); }
    friend Known operator/(const Known& a, const Known& b) { return Known(a.v_ / b.v_, a.s_ / b.s_); }
    template <class A, class = typename std::enable_if<std::is_arithmetic<A>::value>::type>
    friend Known operator+(const Known& a, A b) { return Known(a.v_ + b, a.s_ + Sym(b)); }
    template <class A, class = typename std::enable_if<std::is_arithmetic<A>::value>::type>
    friend Known operator+(A b, const Known& a) { return Known(b + a.v_, Sym(b) + a.s_); }
    template <class A, class = typename std::enable_if<std::is_arithmetic<A>::value>::type>
    friend Known operator-(const Known& a, A b) { return Known(a.v_ - b, a.s_ - Sym(b)); }
    template <class A, class = typename std::enable_if<std::is_arithmetic<A>::value>::type>
    friend Known operator-(A b, const Known& a) { return Known(b - a.v_, Sym(b) - a.s_); }
    template <class A, class = typename std::enable_if<std::is_arithmetic<A>::value>::type>
    friend Known operator*(const Known& a, A b) { return Known(a.v_ * b, a.s_ * Sym(b)); }
    template <class A, class = typename std::enable_if<std::is_arithmetic<A>::value>::type>
    friend Known operator*(A b, const Known& a) { return Known(b * a.v_, Sym(b) * a.s_); }
    template <class A, class = typename std::enable_if<std::is_arithmetic<A>::value>::type>
    friend Known operator/(const Known& a, A b) { return Known(a.v_ / b, a.s_ / Sym(b)); }
    template <class A, class = typename std::enable_if<std::is_arithmetic<A>::value>::type>
    friend Known operator/(A b, const Known& a) { return Known(b / a.v_, Sym(b) / a.s_); }

private:
    double v_;
    Sym s_;
};

// Sym combined with Known keeps the symbol.
inline Sym operator+(const Sym& a, const Known& b) { return a + b.sym(); }
inline Sym operator+(const Known& a, const Sym& b) { return a.sym() + b; }
inline Sym operator-(const Sym& a, const Known& b) { return a - b.sym(); }
inline Sym operator-(const Known& a, const Sym& b) { return a.sym() - b; }
inline Sym operator*(const Sym& a, const Known& b) { return a * b.sym(); }
inline Sym operator*(const Known& a, const Sym& b) { return a.sym() * b; }
inline Sym operator/(const Sym& a, const Known& b) { return a / b.sym(); }

}  // namespace gpu
}  // namespace ScaFES
#endif
