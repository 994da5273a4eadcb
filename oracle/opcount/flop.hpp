// flop.hpp -- TEST INFRASTRUCTURE: an operation-counting stand-in for double.
//
// Force-included (g++ -include) before the oracle's C sources compiled as
// C++: every `double` in them becomes flop_t, whose arithmetic counts one
// operation per + - * / and sqrt, and one transcendental per libm call
// (exp, log, sin, cos, tan, atan, atan2, asin, pow, fmod).  Comparisons,
// negation, fabs, fmin/fmax and conversions are free.  Values are computed
// in plain double, so results stay identical to the normal build.
#pragma once
#include <math.h>
#include <pthread.h>
#include <stddef.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <atomic>
#include <cmath>
#include <cstddef>
#include <cstdlib>

// Per-class counts: add/sub, mul, div, sqrt, then one slot per libm function.
enum FlopClass { FC_ADD, FC_MUL, FC_DIV, FC_SQRT, FC_EXP, FC_LOG, FC_SIN, FC_COS, FC_TAN, FC_ATAN, FC_ASIN,
                 FC_ATAN2, FC_POW, FC_FMOD, FC_N };
struct FlopTally {
    uint64_t ops = 0, trans = 0;
    uint64_t by_class[FC_N] = {0};
};
extern thread_local FlopTally g_tally;

struct flop_t {
    double v;
    flop_t() = default;
    constexpr flop_t(double x) : v(x) {}
    constexpr flop_t(float x) : v(x) {}
    constexpr flop_t(int x) : v(x) {}
    constexpr flop_t(unsigned x) : v(x) {}
    constexpr flop_t(long x) : v((double)x) {}
    constexpr flop_t(unsigned long x) : v((double)x) {}
    constexpr flop_t(long long x) : v((double)x) {}
    constexpr flop_t(unsigned long long x) : v((double)x) {}
    explicit operator int() const { return (int)v; }
    explicit operator long() const { return (long)v; }
    explicit operator long long() const { return (long long)v; }
    explicit operator unsigned long() const { return (unsigned long)v; }
    explicit operator double() const { return v; }
    explicit operator bool() const { return v != 0.0; }
    flop_t operator-() const { return flop_t(-v); }
    flop_t operator+() const { return *this; }
    flop_t& operator+=(flop_t o) { g_tally.ops++; g_tally.by_class[FC_ADD]++; v = v + o.v; return *this; }
    flop_t& operator-=(flop_t o) { g_tally.ops++; g_tally.by_class[FC_ADD]++; v = v - o.v; return *this; }
    flop_t& operator*=(flop_t o) { g_tally.ops++; g_tally.by_class[FC_MUL]++; v = v * o.v; return *this; }
    flop_t& operator/=(flop_t o) { g_tally.ops++; g_tally.by_class[FC_DIV]++; v = v / o.v; return *this; }
};
static_assert(sizeof(flop_t) == 8, "layout must match double");

inline flop_t operator+(flop_t a, flop_t b) { g_tally.ops++; g_tally.by_class[FC_ADD]++; return flop_t(a.v + b.v); }
inline flop_t operator-(flop_t a, flop_t b) { g_tally.ops++; g_tally.by_class[FC_ADD]++; return flop_t(a.v - b.v); }
inline flop_t operator*(flop_t a, flop_t b) { g_tally.ops++; g_tally.by_class[FC_MUL]++; return flop_t(a.v * b.v); }
inline flop_t operator/(flop_t a, flop_t b) { g_tally.ops++; g_tally.by_class[FC_DIV]++; return flop_t(a.v / b.v); }
inline bool operator<(flop_t a, flop_t b) { return a.v < b.v; }
inline bool operator>(flop_t a, flop_t b) { return a.v > b.v; }
inline bool operator<=(flop_t a, flop_t b) { return a.v <= b.v; }
inline bool operator>=(flop_t a, flop_t b) { return a.v >= b.v; }
inline bool operator==(flop_t a, flop_t b) { return a.v == b.v; }
inline bool operator!=(flop_t a, flop_t b) { return a.v != b.v; }

inline flop_t sqrt(flop_t a) { g_tally.ops++; g_tally.by_class[FC_SQRT]++; return flop_t(std::sqrt(a.v)); }
inline flop_t fabs(flop_t a) { return flop_t(std::fabs(a.v)); }
inline flop_t fmin(flop_t a, flop_t b) { return flop_t(std::fmin(a.v, b.v)); }
inline flop_t fmax(flop_t a, flop_t b) { return flop_t(std::fmax(a.v, b.v)); }
inline flop_t round(flop_t a) { return flop_t(std::round(a.v)); }
#define FLOP_T1(fn, cls) \
    inline flop_t fn(flop_t a) { g_tally.trans++; g_tally.by_class[cls]++; return flop_t(std::fn(a.v)); }
FLOP_T1(exp, FC_EXP) FLOP_T1(log, FC_LOG) FLOP_T1(sin, FC_SIN) FLOP_T1(cos, FC_COS) FLOP_T1(tan, FC_TAN)
FLOP_T1(atan, FC_ATAN) FLOP_T1(asin, FC_ASIN)
#undef FLOP_T1
inline flop_t atan2(flop_t a, flop_t b) { g_tally.trans++; g_tally.by_class[FC_ATAN2]++; return flop_t(std::atan2(a.v, b.v)); }
inline flop_t pow(flop_t a, flop_t b) { g_tally.trans++; g_tally.by_class[FC_POW]++; return flop_t(std::pow(a.v, b.v)); }
inline flop_t fmod(flop_t a, flop_t b) { g_tally.trans++; g_tally.by_class[FC_FMOD]++; return flop_t(std::fmod(a.v, b.v)); }
inline int isfinite(flop_t a) { return std::isfinite(a.v); }

#define double flop_t
