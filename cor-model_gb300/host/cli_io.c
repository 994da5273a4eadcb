/*
 * cli_io.c -- INFILE and output formats of `cor -m cutoff`, as in src/io.c:
 * the same fscanf/fprintf formats, so files read and written by the reference
 * are read and written here unchanged.
 */
#include "cli.h"

int read_cutoff_infile_header(FILE *f, InfileHeader *h) {
    /* src/io.c:4-20 */
    const int items = fscanf(f, "%lf %lf %lf\n%lf %lf %lf\n%lf %lf\n%d %d %d %d %d %d %d\n%d %d %d %lf", &h->rig,
                             &h->zn, &h->rk, &h->r0, &h->the0, &h->fi0, &h->the1, &h->fi1, &h->iy, &h->mes, &h->ide,
                             &h->id, &h->ih, &h->min, &h->is, &h->nk1, &h->iopt, &h->ist, &h->del);
    /* The reference rejects only an empty file (items < 0); a header cut short
     * leaves the rest of its stack struct unset and what follows depends on
     * that memory.  Here every one of the 19 items is required. */
    return items != 19 ? -1 : 0;
}

int write_cutoff_outfile_header(FILE *out, const InfileHeader *h, const Model **models, uint64_t steps_count) {
    /* src/io.c:22-50 */
    if (fprintf(out, "\n\n\n                ASYMPTOTIC COORDINATES\n   calculated by model(s): ") < 0) return -1;
    const char *pad = "";
    for (int i = 0; models[i]; i++) {
        if (fprintf(out, "%s%s", pad, models[i]->name) < 0) return -1;
        pad = ", ";
    }
    const int res = fprintf(out,
                            "\n Station with geo.latitude:%9.3f  & longitude:%9.3f & radius : %8.5f\n"
                            " Direction of trajectory with latitude: %9.3f & longitude: %9.3f\n"
                            " Date: %4d %2d %2d  time: %2d hod %2d min %2d sec\n"
                            " Starting rigidity : %8.4f GV Epsilon=%7.4f\n Limit of total number of steps : %lu \n\n"
                            " rig : v : rad : eth : efi : ath : afi : time : length\n",
                            h->the0, h->fi0, h->r0, h->the1, h->fi1, h->iy, h->mes, h->ide, h->ih, h->min, h->is,
                            h->rig, h->del, (unsigned long)steps_count);
    return res < 0 ? -1 : 0;
}

int read_ts05_params(FILE *f, ModelsParams *p) {
    /* src/io.c:98-113: Dst Pdyn By Bz / W1..W6 */
    const int items = fscanf(f, "%lf %lf %lf %lf\n%lf %lf %lf %lf %lf %lf\n", &p->parmod[1], &p->parmod[0],
                             &p->parmod[2], &p->parmod[3], &p->parmod[4], &p->parmod[5], &p->parmod[6],
                             &p->parmod[7], &p->parmod[8], &p->parmod[9]);
    return items != 10 ? -1 : 0;
}

int read_t96_params(FILE *f, ModelsParams *p) {
    /* src/io.c:115-127: Dst Pdyn By Bz */
    const int items = fscanf(f, "%lf %lf %lf %lf\n", &p->parmod[1], &p->parmod[0], &p->parmod[2], &p->parmod[3]);
    return items != 4 ? -1 : 0;
}

int read_field_infile_header(FILE *f, InfileHeader *h) {
    /* src/io.c:52-67: r0 lat0 lon0 / lat_step lon_step lat1 lon1 / date */
    const int items = fscanf(f, "%lf %lf %lf\n%lf %lf %lf %lf\n%d %d %d %d %d %d %d\n", &h->r0, &h->the0, &h->fi0,
                             &h->lat_step, &h->lon_step, &h->the1, &h->fi1, &h->iy, &h->mes, &h->ide, &h->id, &h->ih,
                             &h->min, &h->is);
    return items != 14 ? -1 : 0;  /* all 14 items, as for the cutoff header */
}

int write_field_outfile_header(FILE *out, const InfileHeader *h, const Model **models) {
    /* src/io.c:69-96 */
    if (fprintf(out, "\n\n\n                GEOMAGNETIC FIELD\n Geomagnetic Model(s): ") < 0) return -1;
    const char *pad = "";
    for (int i = 0; models[i]; i++) {
        if (fprintf(out, "%s%s", pad, models[i]->name) < 0) return -1;
        pad = ", ";
    }
    const int res = fprintf(out,
                            "\n lat step: %.3f, lon step: %.3f\n"
                            " Date: %4d %2d %2d  time: %2d h %2d min %2d sec\n\n"
                            " lat : lon : B [nT] : BXGEO [nT] : BYGEO [nT] : BZGEO [nT]\n",
                            h->lat_step, h->lon_step, h->iy, h->mes, h->ide, h->ih, h->min, h->is);
    return res < 0 ? -1 : 0;
}
