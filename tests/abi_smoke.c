/*
 * abi_smoke.c -- a plain C caller of include/lulesh_gb300.h, linked against
 * liblulesh_gb300.so the way a C or C++ host program links it (no Python).
 *
 *   abi_smoke run  NX NUMREG BALANCE COST ITS PRECISION OUTDIR
 *       lg_create -> lg_run -> lg_verify / lg_report / lg_get_field, as the
 *       reference's main() does with Domain, the cycle loop and
 *       VerifyAndWriteFinalOutput (lulesh.cc:2715-2767, lulesh-util.cc:175-230).
 *       Prints "status", "cycle", "time", "verify" lines and the report text,
 *       and writes every double accessor field to OUTDIR/<name>.f64.
 *
 *   abi_smoke sync NX NUMREG BALANCE COST NCYCLES PRECISION
 *       The second integration pattern: the caller keeps every Domain field
 *       in its own host arrays and, around every cycle, uploads all of them
 *       (lg_set_field), runs lg_step(1) and downloads all of them
 *       (lg_get_field).  A second handle runs the same cycles with the state
 *       resident.  Prints "sync-equal 1" when both end bit for bit equal.
 *
 * Exit status 0 on success; any API error prints lg_last_error() and exits 1.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "lulesh_gb300.h"

static const char *const NODE_FIELDS[] = {"x",  "y",  "z",  "xd", "yd", "zd", "xdd",
                                          "ydd", "zdd", "fx", "fy", "fz", "nodalMass"};
static const char *const ELEM_FIELDS[] = {"e",    "p",    "q",    "ql",     "qq", "v",
                                          "volo", "vnew", "delv", "vdov", "arealg", "ss",
                                          "elemMass"};
#define NFIELDS 13

static void check(int st, const char *what)
{
    if (st > 0) {
        fprintf(stderr, "%s failed (%d): %s\n", what, st, lg_last_error());
        exit(1);
    }
}

static int parse_precision(const char *s)
{
    if (!strcmp(s, "fp64")) return LG_FP64;
    if (!strcmp(s, "fp64-fma")) return LG_FP64_FMA;
    if (!strcmp(s, "mixed")) return LG_MIXED;
    fprintf(stderr, "unknown precision %s\n", s);
    exit(2);
}

static lg_domain *create(char **argv)
{
    lg_opts o;
    lg_default_opts(&o);
    o.nx = atoi(argv[0]);
    o.numReg = atoi(argv[1]);
    o.balance = atoi(argv[2]);
    o.cost = atoi(argv[3]);
    o.its = atoi(argv[4]);
    o.precision = parse_precision(argv[5]);
    lg_domain *d = NULL;
    check(lg_create(&o, &d), "lg_create");
    return d;
}

static size_t field_len(lg_domain *d, const char *name)
{
    size_t n = 0;
    int dtype = -1;
    check(lg_field_info(d, name, &n, &dtype), "lg_field_info");
    if (dtype != LG_F64) {
        fprintf(stderr, "%s is not a double field\n", name);
        exit(1);
    }
    return n;
}

static int cmd_run(char **argv)
{
    lg_domain *d = create(argv);
    const char *outdir = argv[6];
    const int st = lg_run(d);
    check(st, "lg_run");
    double cycle = 0, time = 0, v[4];
    check(lg_get_scalar(d, "cycle", &cycle), "lg_get_scalar(cycle)");
    check(lg_get_scalar(d, "time", &time), "lg_get_scalar(time)");
    check(lg_verify(d, v), "lg_verify");
    printf("status %d\ncycle %.0f\ntime %.17g\n", st, cycle, time);
    printf("verify %.17g %.17g %.17g %.17g\n", v[0], v[1], v[2], v[3]);
    char report[8192];
    check(lg_report(d, 1.0, report, sizeof report), "lg_report");
    printf("--- report\n%s--- end\n", report);
    for (int k = 0; k < 2; ++k) {
        const char *const *names = k ? ELEM_FIELDS : NODE_FIELDS;
        for (int i = 0; i < NFIELDS; ++i) {
            const size_t n = field_len(d, names[i]);
            double *buf = malloc(n * sizeof(double));
            if (!buf) return 1;
            check(lg_get_field(d, names[i], buf, n), "lg_get_field");
            char path[4096];
            snprintf(path, sizeof path, "%s/%s.f64", outdir, names[i]);
            FILE *f = fopen(path, "wb");
            if (!f || fwrite(buf, sizeof(double), n, f) != n) {
                fprintf(stderr, "cannot write %s\n", path);
                return 1;
            }
            fclose(f);
            free(buf);
        }
    }
    lg_destroy(d);
    return 0;
}

static int cmd_sync(char **argv)
{
    const int ncycles = atoi(argv[4]);
    char *args[6] = {argv[0], argv[1], argv[2], argv[3], "9999999", argv[5]};
    lg_domain *resident = create(args);
    lg_domain *synced = create(args);
    /* the caller's host copy of every field, starting from the set-up state */
    double *host[2][NFIELDS];
    size_t len[2][NFIELDS];
    for (int k = 0; k < 2; ++k)
        for (int i = 0; i < NFIELDS; ++i) {
            const char *name = k ? ELEM_FIELDS[i] : NODE_FIELDS[i];
            len[k][i] = field_len(synced, name);
            host[k][i] = malloc(len[k][i] * sizeof(double));
            if (!host[k][i]) return 1;
            check(lg_get_field(synced, name, host[k][i], len[k][i]), "lg_get_field");
        }
    for (int c = 0; c < ncycles; ++c) {
        for (int k = 0; k < 2; ++k)
            for (int i = 0; i < NFIELDS; ++i)
                check(lg_set_field(synced, k ? ELEM_FIELDS[i] : NODE_FIELDS[i], host[k][i],
                                   len[k][i]), "lg_set_field");
        check(lg_step(synced, 1), "lg_step(synced)");
        for (int k = 0; k < 2; ++k)
            for (int i = 0; i < NFIELDS; ++i)
                check(lg_get_field(synced, k ? ELEM_FIELDS[i] : NODE_FIELDS[i], host[k][i],
                                   len[k][i]), "lg_get_field");
    }
    check(lg_step(resident, ncycles), "lg_step(resident)");
    int equal = 1;
    for (int k = 0; k < 2; ++k)
        for (int i = 0; i < NFIELDS; ++i) {
            const char *name = k ? ELEM_FIELDS[i] : NODE_FIELDS[i];
            double *buf = malloc(len[k][i] * sizeof(double));
            if (!buf) return 1;
            check(lg_get_field(resident, name, buf, len[k][i]), "lg_get_field");
            if (memcmp(buf, host[k][i], len[k][i] * sizeof(double))) {
                printf("differs: %s\n", name);
                equal = 0;
            }
            free(buf);
            free(host[k][i]);
        }
    double c1 = 0, c2 = 0;
    check(lg_get_scalar(resident, "cycle", &c1), "lg_get_scalar");
    check(lg_get_scalar(synced, "cycle", &c2), "lg_get_scalar");
    printf("cycles %.0f %.0f\nsync-equal %d\n", c1, c2, equal && c1 == c2);
    lg_destroy(resident);
    lg_destroy(synced);
    return 0;
}

int main(int argc, char **argv)
{
    if (argc == 9 && !strcmp(argv[1], "run")) return cmd_run(argv + 2);
    if (argc == 8 && !strcmp(argv[1], "sync")) return cmd_sync(argv + 2);
    fprintf(stderr,
            "usage: %s run NX NUMREG BALANCE COST ITS PRECISION OUTDIR\n"
            "       %s sync NX NUMREG BALANCE COST NCYCLES PRECISION\n",
            argv[0], argv[0]);
    return 2;
}
