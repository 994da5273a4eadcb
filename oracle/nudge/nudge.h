/*
 * nudge.h -- TEST INFRASTRUCTURE: one-ulp libm perturbation of the oracle.
 *
 * Force-included (gcc -include) into the oracle's C sources to build
 * liboracle_nudge.so: every call of exp, log, sin, cos, tan, atan, atan2,
 * asin and pow returns the C library's result moved by one ulp up or down
 * (a seeded per-thread pseudo-random sign).  The spread this causes in the
 * oracle's own results measures how sensitive the reference's algorithm is
 * to a one-ulp difference in its math library -- the yardstick for a GPU
 * whose FP64 transcendentals differ from the C library's by a few ulp.
 */
#ifndef COR_NUDGE_H
#define COR_NUDGE_H
#include <math.h>
#include <stdint.h>

double orc_nudge(double v);
void orc_nudge_seed(uint64_t seed);

#define exp(x) orc_nudge(__builtin_exp(x))
#define log(x) orc_nudge(__builtin_log(x))
#define sin(x) orc_nudge(__builtin_sin(x))
#define cos(x) orc_nudge(__builtin_cos(x))
#define tan(x) orc_nudge(__builtin_tan(x))
#define atan(x) orc_nudge(__builtin_atan(x))
#define asin(x) orc_nudge(__builtin_asin(x))
#define atan2(y, x) orc_nudge(__builtin_atan2((y), (x)))
#define pow(x, y) orc_nudge(__builtin_pow((x), (y)))
#endif
