/*
 * tlq_oracle_count.cpp -- the oracle (tlq_oracle.c) compiled a second time
 * with every double replaced by a counting double, to count the FP64
 * operations of the reference algorithm per zone-update.
 *
 * TEST AND MEASUREMENT INFRASTRUCTURE ONLY (like the oracle itself): never
 * linked or called by the product.  The counted type holds one double and
 * performs each operation once, in IEEE double with the same evaluation
 * order, so this build computes exactly the oracle's numbers (a test checks
 * that, bit for bit); it only adds a counter to every operation.  Serial:
 * built without OpenMP, so the counters need no atomics.
 *
 * Categories: add (+ and - of two values, including compound assignment),
 * mul, div, sqrt, cmp (<, >, <=, >=, ==, !=, which also carry the Fortran
 * MIN/MAX), trans (exp, log, log10, pow, and the self-gravity's acos, atan2, cos,
 * sin, Gamma); fabs, copysign, ceil, negation and conversions are not
 * counted.
 */
#include <cmath>
#include <cstdlib>
#include <cstring>

namespace {
unsigned long long g_add, g_mul, g_div, g_sqrt, g_cmp, g_trans;
}

struct fd {
  double v;
  fd() = default;
  constexpr fd(double x) : v(x) {}
  explicit operator long() const { return (long)v; }
  explicit operator int() const { return (int)v; }
  explicit operator unsigned() const { return (unsigned)v; }
  explicit operator bool() const { return v != 0.0; }
  fd& operator+=(fd b) { ++g_add; v += b.v; return *this; }
  fd& operator-=(fd b) { ++g_add; v -= b.v; return *this; }
  fd& operator*=(fd b) { ++g_mul; v *= b.v; return *this; }
  fd& operator/=(fd b) { ++g_div; v /= b.v; return *this; }
};
static_assert(sizeof(fd) == sizeof(double) && alignof(fd) == alignof(double), "fd is laid out as a double");

inline fd operator+(fd a, fd b) { ++g_add; return fd(a.v + b.v); }
inline fd operator-(fd a, fd b) { ++g_add; return fd(a.v - b.v); }
inline fd operator*(fd a, fd b) { ++g_mul; return fd(a.v * b.v); }
inline fd operator/(fd a, fd b) { ++g_div; return fd(a.v / b.v); }
inline fd operator-(fd a) { return fd(-a.v); }
inline fd operator+(fd a) { return a; }
inline bool operator<(fd a, fd b) { ++g_cmp; return a.v < b.v; }
inline bool operator>(fd a, fd b) { ++g_cmp; return a.v > b.v; }
inline bool operator<=(fd a, fd b) { ++g_cmp; return a.v <= b.v; }
inline bool operator>=(fd a, fd b) { ++g_cmp; return a.v >= b.v; }
inline bool operator==(fd a, fd b) { ++g_cmp; return a.v == b.v; }
inline bool operator!=(fd a, fd b) { ++g_cmp; return a.v != b.v; }
inline fd sqrt(fd a) { ++g_sqrt; return fd(std::sqrt(a.v)); }
inline fd exp(fd a) { ++g_trans; return fd(std::exp(a.v)); }
inline fd log10(fd a) { ++g_trans; return fd(std::log10(a.v)); }
inline fd log(fd a) { ++g_trans; return fd(std::log(a.v)); }
inline fd pow(fd a, fd b) { ++g_trans; return fd(std::pow(a.v, b.v)); }
inline fd fabs(fd a) { return fd(std::fabs(a.v)); }
inline fd copysign(fd a, fd b) { return fd(std::copysign(a.v, b.v)); }
inline fd ceil(fd a) { return fd(std::ceil(a.v)); }
inline fd acos(fd a) { ++g_trans; return fd(std::acos(a.v)); }
inline fd atan2(fd a, fd b) { ++g_trans; return fd(std::atan2(a.v, b.v)); }
inline fd cos(fd a) { ++g_trans; return fd(std::cos(a.v)); }
inline fd sin(fd a) { ++g_trans; return fd(std::sin(a.v)); }
inline fd tgamma(fd a) { ++g_trans; return fd(std::tgamma(a.v)); }

// Every header the oracle includes is included above, before the macro, so
// that only the oracle's own code sees it.
#define double fd
#include "tlq_oracle.c"
#undef double

extern "C" {

/* Operation counts since the last reset. */
typedef struct tlqo_flops {
  double add, mul, div, sqrt, cmp, trans;
} tlqo_flops;

void tlqo_flops_reset(void) { g_add = g_mul = g_div = g_sqrt = g_cmp = g_trans = 0; }

void tlqo_flops_get(tlqo_flops* out) {
  out->add = (double)g_add;
  out->mul = (double)g_mul;
  out->div = (double)g_div;
  out->sqrt = (double)g_sqrt;
  out->cmp = (double)g_cmp;
  out->trans = (double)g_trans;
}

}  // extern "C"
