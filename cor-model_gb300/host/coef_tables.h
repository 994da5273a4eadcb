/* Coefficient tables of the field models (data in coef_tables.c). */
#ifndef COR_COEF_TABLES_H
#define COR_COEF_TABLES_H

/* One internal model: the epoch list of InternalModelCoefs
 * (lib/internal/coefs/coefs.h:8-15).  gh[2k] / gh[2k+1] are G / H of epoch k,
 * epochs years_step apart from min_year; for extrapolating models the last
 * pair holds the secular variation [nT/yr]. */
typedef struct {
    const char *version;   /* -i name, src/models.c:24 ... */
    const char *name;      /* printed model name          */
    const double *const *gh;
    int n_arrays;
    int years_step;
    int min_year;
    int max_year;
    int extrapolate;
} cor_sh_table;

/* Lithospheric table: G and H packed as the lower triangle, index n*(n+1)/2+m. */
typedef struct {
    const char *version;
    const char *name;
    int nmax;
    const double *g;
    const double *h;
} cor_chaos_table;

extern const cor_sh_table cor_sh_tables[];
extern const int cor_sh_table_count;
extern const cor_chaos_table cor_chaos716;

#endif
