/*
 * orc_flops.cpp -- the oracle with its floating-point operations counted.
 *
 * TEST INFRASTRUCTURE ONLY (see fjoracle.h).  The oracle's C sources
 * (orc_numerics.c, orc_model.c: the reference's algorithm restated) are
 * compiled here with `double` replaced by a type that performs the same IEEE
 * double arithmetic and tallies each operation, so the results are the
 * oracle's bit for bit and the tally is the algorithm's work, independent of
 * how any implementation schedules it:
 *   add   additions and subtractions      mul   multiplications
 *   div   divisions                       sqrt  square roots
 *   trans calls of exp, log10, pow, sin, cos, sinh, cosh, tanh, asinh,
 *         acos, asin, atan2 (weighted when summed, see orc_flops_get)
 * Comparisons, fabs, negation and conversions are not counted.  Built as
 * liboracle_flops.so with the same C entry points as liboracle.so plus
 * orc_flops_reset / orc_flops_get; the tally is per host thread.
 */
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <type_traits>
#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

namespace fjc {
struct Tally {
    unsigned long long add = 0, mul = 0, div = 0, sqrt = 0, trans = 0;
};
inline Tally &tally()
{
    static thread_local Tally t;
    return t;
}

struct D {
    double v;
    D() = default;
    constexpr D(double x) : v(x) {}
    template <class I, class = typename std::enable_if<std::is_integral<I>::value>::type>
    constexpr D(I x) : v((double)x) {}
    explicit operator double() const { return v; }
    explicit operator float() const { return (float)v; }
    template <class I, class = typename std::enable_if<std::is_integral<I>::value>::type>
    explicit operator I() const { return (I)v; }
    explicit operator bool() const { return v != 0; }
    D &operator+=(D o) { tally().add++; v += o.v; return *this; }
    D &operator-=(D o) { tally().add++; v -= o.v; return *this; }
    D &operator*=(D o) { tally().mul++; v *= o.v; return *this; }
    D &operator/=(D o) { tally().div++; v /= o.v; return *this; }
};
static_assert(sizeof(D) == sizeof(double) && std::is_trivially_copyable<D>::value, "D must be laid out as a double");
inline D operator+(D a, D b) { tally().add++; return D(a.v + b.v); }
inline D operator-(D a, D b) { tally().add++; return D(a.v - b.v); }
inline D operator*(D a, D b) { tally().mul++; return D(a.v * b.v); }
inline D operator/(D a, D b) { tally().div++; return D(a.v / b.v); }
inline D operator-(D a) { return D(-a.v); }
inline D operator+(D a) { return a; }
inline bool operator<(D a, D b) { return a.v < b.v; }
inline bool operator>(D a, D b) { return a.v > b.v; }
inline bool operator<=(D a, D b) { return a.v <= b.v; }
inline bool operator>=(D a, D b) { return a.v >= b.v; }
inline bool operator==(D a, D b) { return a.v == b.v; }
inline bool operator!=(D a, D b) { return a.v != b.v; }
}  // namespace fjc

using fjc::D;
inline D sqrt(D x) { fjc::tally().sqrt++; return std::sqrt(x.v); }
inline D fabs(D x) { return std::fabs(x.v); }
inline int isnan(D x) { return std::isnan(x.v); }
#define FJC_T1(f) \
    inline D f(D x) { fjc::tally().trans++; return std::f(x.v); }
FJC_T1(exp) FJC_T1(log10) FJC_T1(sin) FJC_T1(cos) FJC_T1(sinh) FJC_T1(cosh) FJC_T1(tanh) FJC_T1(asinh)
FJC_T1(acos) FJC_T1(asin)
#undef FJC_T1
inline D pow(D a, D b) { fjc::tally().trans++; return std::pow(a.v, b.v); }
inline D atan2(D a, D b) { fjc::tally().trans++; return std::atan2(a.v, b.v); }

#define _Thread_local thread_local
#define double D
#include "orc_numerics.c"
#include "orc_model.c"
#undef double

extern "C" {
void orc_flops_reset(void) { fjc::tally() = fjc::Tally(); }
/* out[0..4] = add, mul, div, sqrt, trans counts of this host thread */
void orc_flops_get(unsigned long long *out)
{
    const fjc::Tally &t = fjc::tally();
    out[0] = t.add; out[1] = t.mul; out[2] = t.div; out[3] = t.sqrt; out[4] = t.trans;
}
}
