// ref_driver.cc -- C entry points around the UNCHANGED reference sources.
//
// TEST INFRASTRUCTURE ONLY.  Compiled by oracle/Makefile against the LULESH
// 2.x sources where they lie (never copied into this repository), with the
// reference main() renamed.  It exposes the reference's own Domain and its
// file-static TimeIncrement / LagrangeLeapFrog (lulesh.cc:166, 2601) so the
// C restatement in lulesh_oracle.c can be checked against the reference
// itself, field by field.  Errors in the reference call exit(), so callers run
// this in a child process.
//
// Standard headers come first so that the access-specifier override below
// only touches class Domain (lulesh.h:148-595); it is needed to vary the
// const member m_hgcoef (lulesh-init.cc:25) for the parameter studies.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctype.h>
#include <iomanip>
#include <iostream>
#include <limits.h>
#include <string.h>
#include <sys/time.h>
#include <time.h>
#include <unistd.h>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#define private public
#include "lulesh.cc"
#undef private

extern "C" {

void *ref_create(int nx, int nr, int balance, int cost, double hgcoef, double einit_factor)
{
#ifdef _OPENMP
    // The corner-gather force path the oracle follows is only taken with
    // more than one thread (lulesh.cc:514, lulesh-init.cc:280).
    if (omp_get_max_threads() < 2) omp_set_num_threads(2);
#endif
    Domain *d = new Domain(1, 0, 0, 0, nx, 1, nr, balance, cost);
    const_cast<Real_t &>(d->m_hgcoef) = hgcoef;
    if (einit_factor != 1.0) {
        // same expression order as lulesh-init.cc:183-192
        const Real_t ebase = Real_t(3.948746e+7);
        Real_t scale = (nx * 1) / Real_t(45.0);
        Real_t einit = ebase * scale * scale * scale;
        einit = einit * einit_factor;
        d->e(0) = einit;
        d->deltatime() = (Real_t(.5) * cbrt(d->volo(0))) / sqrt(Real_t(2.0) * einit);
    }
    return d;
}

void ref_destroy(void *h) { delete static_cast<Domain *>(h); }

// The reference main loop, lulesh.cc:2745-2757, for at most ncycles cycles.
int ref_step(void *h, int ncycles)
{
    Domain &d = *static_cast<Domain *>(h);
    for (int c = 0; c < ncycles && d.time() < d.stoptime(); ++c) {
        TimeIncrement(d);
        LagrangeLeapFrog(d);
    }
    return d.cycle();
}

// The main loop with the time steps given: cycle c advances by dts[c]
// instead of TimeIncrement's choice (the bookkeeping of lulesh.cc:218-221),
// then LagrangeLeapFrog.
int ref_step_frozen(void *h, const double *dts, int ncycles)
{
    Domain &d = *static_cast<Domain *>(h);
    for (int c = 0; c < ncycles; ++c) {
        d.deltatime() = dts[c];
        d.time() += d.deltatime();
        ++d.cycle();
        LagrangeLeapFrog(d);
    }
    return d.cycle();
}

double *ref_field_f64(void *h, const char *name, size_t *n)
{
    Domain &d = *static_cast<Domain *>(h);
    const size_t N = d.numNode(), E = d.numElem();
    struct { const char *nm; double *p; size_t len; } t[] = {
        {"x", &d.x(0), N}, {"y", &d.y(0), N}, {"z", &d.z(0), N},
        {"xd", &d.xd(0), N}, {"yd", &d.yd(0), N}, {"zd", &d.zd(0), N},
        {"xdd", &d.xdd(0), N}, {"ydd", &d.ydd(0), N}, {"zdd", &d.zdd(0), N},
        {"fx", &d.fx(0), N}, {"fy", &d.fy(0), N}, {"fz", &d.fz(0), N},
        {"nodalMass", &d.nodalMass(0), N},
        {"e", &d.e(0), E}, {"p", &d.p(0), E}, {"q", &d.q(0), E},
        {"ql", &d.ql(0), E}, {"qq", &d.qq(0), E}, {"v", &d.v(0), E},
        {"volo", &d.volo(0), E}, {"vnew", &d.vnew(0), E}, {"delv", &d.delv(0), E},
        {"vdov", &d.vdov(0), E}, {"arealg", &d.arealg(0), E}, {"ss", &d.ss(0), E},
        {"elemMass", &d.elemMass(0), E}};
    for (auto &f : t)
        if (!strcmp(f.nm, name)) {
            if (n) *n = f.len;
            return f.p;
        }
    return nullptr;
}

int *ref_field_i32(void *h, const char *name, size_t *n)
{
    Domain &d = *static_cast<Domain *>(h);
    const size_t E = d.numElem();
    if (!strcmp(name, "regNumList")) { if (n) *n = E; return d.regNumList(); }
    if (!strcmp(name, "nodelist")) { if (n) *n = 8 * E; return d.nodelist(0); }
    if (!strcmp(name, "elemBC")) { if (n) *n = E; return &d.elemBC(0); }
    return nullptr;
}

double ref_get_scalar(void *h, const char *name)
{
    Domain &d = *static_cast<Domain *>(h);
    if (!strcmp(name, "time")) return d.time();
    if (!strcmp(name, "deltatime")) return d.deltatime();
    if (!strcmp(name, "dtcourant")) return d.dtcourant();
    if (!strcmp(name, "dthydro")) return d.dthydro();
    if (!strcmp(name, "cycle")) return d.cycle();
    if (!strcmp(name, "hgcoef")) return d.hgcoef();
    return NAN;
}

// Replace the energy field before the run (perturbed initial energies).
void ref_set_e(void *h, const double *e, size_t n)
{
    Domain &d = *static_cast<Domain *>(h);
    for (size_t i = 0; i < n && i < (size_t)d.numElem(); ++i) d.e(i) = e[i];
}

// The reference's end-of-run report (lulesh-util.cc:175-230).
void ref_report(void *h, double elapsed, int nx)
{
    Domain &d = *static_cast<Domain *>(h);
    VerifyAndWriteFinalOutput(elapsed, d, nx, 1);
    std::cout.flush();
}

}  // extern "C"
