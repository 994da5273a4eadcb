/*
 * external_pending.c -- TEST INFRASTRUCTURE, not part of the product.
 * Placeholder for the TS05 restatement: returns NaN so that any
 * comparison against it fails loudly until the restatement lands.
 */
#include "cor_oracle.h"
#include <math.h>

void orc_ts05_gsm(const double *parmod, double x, double y, double z, double *bx, double *by, double *bz) {
    (void)parmod; (void)x; (void)y; (void)z;
    *bx = *by = *bz = NAN;
}
