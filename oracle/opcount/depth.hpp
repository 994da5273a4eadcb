// depth.hpp -- TEST INFRASTRUCTURE: a dependency-depth-tracking stand-in for
// double, for measuring how much of one accepted step's work could run at
// once (oracle/opcount/critical_path.py).
//
// Force-included (g++ -include) before the oracle's C sources compiled as
// C++: every `double` in them becomes dep_t, which carries its value and the
// length of the longest chain of dependent operations that produced it.
// Every operation adds its latency to the deeper of its operands; a
// comparison raises a thread-wide control floor to the depth of what it
// compared, and every later result starts from at least that floor, so work
// after a branch waits for the branch's condition, as a single thread's must.
// Latencies are in units of one dependent FP64 add/mul/FMA; divisions, square
// roots and C-library functions take the weights below, and the same weights
// give each operation's issue cost (the FP64 instructions it takes).  Values
// are computed in plain double, so results stay identical to the normal build.
#pragma once
#include <math.h>
#include <pthread.h>
#include <stddef.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdlib>

typedef double raw_double;   // the plain type, for reading ABI structs from files

// Dependent-operation latency and issue cost of each operation class, in
// units of one FP64 add/mul/FMA.  Division and square root: the measured
// latencies of one dependent sequence on this GPU (562 and 678 cycles against
// 64 for an FMA) and about 9 and 10 FP64 instructions each; a C-library
// function: 20 dependent operations and 20 instructions (the weight of the
// work model).
struct DepWeights {
    double lat_div = 562. / 64., lat_sqrt = 678. / 64., lat_trans = 20.;
    double issue_div = 9., issue_sqrt = 10., issue_trans = 20.;
};
struct DepTally {
    double floor = 0.;   // control floor: depth of the latest branch condition
    double max = 0.;     // deepest result so far
    double issue = 0.;   // FP64 instructions issued
    uint64_t ops = 0;
};
extern thread_local DepTally g_dep;
extern const DepWeights g_w;

struct dep_t {
    double v;
    double d;
    dep_t() = default;
    constexpr dep_t(double x) : v(x), d(0.) {}
    constexpr dep_t(float x) : v(x), d(0.) {}
    constexpr dep_t(int x) : v(x), d(0.) {}
    constexpr dep_t(unsigned x) : v(x), d(0.) {}
    constexpr dep_t(long x) : v((double)x), d(0.) {}
    constexpr dep_t(unsigned long x) : v((double)x), d(0.) {}
    constexpr dep_t(long long x) : v((double)x), d(0.) {}
    constexpr dep_t(unsigned long long x) : v((double)x), d(0.) {}
    constexpr dep_t(double x, double depth) : v(x), d(depth) {}
    explicit operator int() const { return (int)v; }
    explicit operator long() const { return (long)v; }
    explicit operator long long() const { return (long long)v; }
    explicit operator unsigned long() const { return (unsigned long)v; }
    explicit operator unsigned() const { return (unsigned)v; }
    explicit operator double() const { return v; }
    explicit operator bool() const { return v != 0.0; }
    dep_t operator-() const { return dep_t(-v, d); }
    dep_t operator+() const { return *this; }
};

inline dep_t dep_op(double v, double da, double db, double lat, double issue) {
    const double d = std::max(std::max(da, db), g_dep.floor) + lat;
    g_dep.max = std::max(g_dep.max, d);
    g_dep.issue += issue;
    g_dep.ops++;
    return dep_t(v, d);
}
inline dep_t operator+(dep_t a, dep_t b) { return dep_op(a.v + b.v, a.d, b.d, 1., 1.); }
inline dep_t operator-(dep_t a, dep_t b) { return dep_op(a.v - b.v, a.d, b.d, 1., 1.); }
inline dep_t operator*(dep_t a, dep_t b) { return dep_op(a.v * b.v, a.d, b.d, 1., 1.); }
inline dep_t operator/(dep_t a, dep_t b) { return dep_op(a.v / b.v, a.d, b.d, g_w.lat_div, g_w.issue_div); }
inline dep_t& operator+=(dep_t& a, dep_t b) { return a = a + b; }
inline dep_t& operator-=(dep_t& a, dep_t b) { return a = a - b; }
inline dep_t& operator*=(dep_t& a, dep_t b) { return a = a * b; }
inline dep_t& operator/=(dep_t& a, dep_t b) { return a = a / b; }

inline bool dep_cmp(bool r, dep_t a, dep_t b) {
    g_dep.floor = std::max(g_dep.floor, std::max(a.d, b.d));
    return r;
}
inline bool operator<(dep_t a, dep_t b) { return dep_cmp(a.v < b.v, a, b); }
inline bool operator>(dep_t a, dep_t b) { return dep_cmp(a.v > b.v, a, b); }
inline bool operator<=(dep_t a, dep_t b) { return dep_cmp(a.v <= b.v, a, b); }
inline bool operator>=(dep_t a, dep_t b) { return dep_cmp(a.v >= b.v, a, b); }
inline bool operator==(dep_t a, dep_t b) { return dep_cmp(a.v == b.v, a, b); }
inline bool operator!=(dep_t a, dep_t b) { return dep_cmp(a.v != b.v, a, b); }

inline dep_t sqrt(dep_t a) { return dep_op(std::sqrt(a.v), a.d, 0., g_w.lat_sqrt, g_w.issue_sqrt); }
inline dep_t fabs(dep_t a) { return dep_t(std::fabs(a.v), a.d); }
inline dep_t fmin(dep_t a, dep_t b) { return dep_op(std::fmin(a.v, b.v), a.d, b.d, 1., 1.); }
inline dep_t fmax(dep_t a, dep_t b) { return dep_op(std::fmax(a.v, b.v), a.d, b.d, 1., 1.); }
inline dep_t round(dep_t a) { return dep_op(std::round(a.v), a.d, 0., 1., 1.); }
#define DEP_T1(fn) \
    inline dep_t fn(dep_t a) { return dep_op(std::fn(a.v), a.d, 0., g_w.lat_trans, g_w.issue_trans); }
DEP_T1(exp) DEP_T1(log) DEP_T1(sin) DEP_T1(cos) DEP_T1(tan) DEP_T1(atan) DEP_T1(asin)
#undef DEP_T1
inline dep_t atan2(dep_t a, dep_t b) { return dep_op(std::atan2(a.v, b.v), a.d, b.d, g_w.lat_trans, g_w.issue_trans); }
inline dep_t pow(dep_t a, dep_t b) { return dep_op(std::pow(a.v, b.v), a.d, b.d, g_w.lat_trans, g_w.issue_trans); }
inline dep_t fmod(dep_t a, dep_t b) { return dep_op(std::fmod(a.v, b.v), a.d, b.d, g_w.lat_trans, g_w.issue_trans); }
inline int isfinite(dep_t a) { return std::isfinite(a.v); }

#define double dep_t
