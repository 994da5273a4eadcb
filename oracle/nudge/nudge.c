/* nudge.c -- TEST INFRASTRUCTURE: the random one-ulp move of nudge.h.
 * Each thread draws from its own xorshift stream, seeded from the global
 * seed and a per-thread counter the first time it perturbs a value. */
#include <math.h>
#include <stdint.h>

static volatile uint64_t g_seed = 1;
static volatile uint64_t g_generation = 1;
static volatile uint64_t g_threads = 0;
static __thread uint64_t t_state = 0, t_generation = 0;

void orc_nudge_seed(uint64_t seed) {
    g_seed = seed;
    __atomic_add_fetch(&g_generation, 1, __ATOMIC_SEQ_CST);
}

double orc_nudge(double v) {
    if (t_generation != g_generation) {
        const uint64_t k = __atomic_add_fetch(&g_threads, 1, __ATOMIC_SEQ_CST);
        t_state = (g_seed * 0x9E3779B97F4A7C15ull) ^ (k * 0xBF58476D1CE4E5B9ull) ^ 0x94D049BB133111EBull;
        t_generation = g_generation;
    }
    t_state ^= t_state << 13;
    t_state ^= t_state >> 7;
    t_state ^= t_state << 17;
    if (!isfinite(v)) return v;
    return nextafter(v, (t_state >> 33) & 1 ? INFINITY : -INFINITY);
}
