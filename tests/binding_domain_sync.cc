// binding_domain_sync.cc -- the second integration pattern as a compilable
// unit: the reference keeps its own Domain (lulesh.h:148-595) on the host and
// hands each stretch of cycles to the GPU path, syncing every accessor field
// and the time-step scalars around it.  tests/test_host.py compiles this file
// against the reference's unchanged lulesh.h (syntax check, no link), so the
// snippet a maintainer copies from the integration guide is known to compile.
#include "lulesh.h"
#include "lulesh_gb300.h"

namespace {

// Accessor name -> Domain member function (Domain_member, lulesh.h:597).
struct FieldBinding {
    const char *name;
    Domain_member get;
};

const FieldBinding kNodeFields[] = {
    {"x", &Domain::x},     {"y", &Domain::y},     {"z", &Domain::z},
    {"xd", &Domain::xd},   {"yd", &Domain::yd},   {"zd", &Domain::zd},
    {"xdd", &Domain::xdd}, {"ydd", &Domain::ydd}, {"zdd", &Domain::zdd},
    {"fx", &Domain::fx},   {"fy", &Domain::fy},   {"fz", &Domain::fz},
    {"nodalMass", &Domain::nodalMass}};

const FieldBinding kElemFields[] = {
    {"e", &Domain::e},       {"p", &Domain::p},           {"q", &Domain::q},
    {"ql", &Domain::ql},     {"qq", &Domain::qq},         {"v", &Domain::v},
    {"volo", &Domain::volo}, {"vnew", &Domain::vnew},     {"delv", &Domain::delv},
    {"vdov", &Domain::vdov}, {"arealg", &Domain::arealg}, {"ss", &Domain::ss},
    {"elemMass", &Domain::elemMass}};

}  // namespace

// Run n cycles of TimeIncrement + LagrangeLeapFrog for `dom` on the GPU
// handle g (created with the same -s -r -b -c options): upload every field
// and the time-step state, step, and copy everything back into dom.
// Returns the lg_step status: 0, -1 (VolumeError), -2 (QStopError) or an
// API error.
int lg_advance_domain(Domain &dom, lg_domain *g, int n)
{
    int st;
    for (const FieldBinding &f : kNodeFields)
        if ((st = lg_set_field(g, f.name, &(dom.*f.get)(0), (size_t)dom.numNode()))) return st;
    for (const FieldBinding &f : kElemFields)
        if ((st = lg_set_field(g, f.name, &(dom.*f.get)(0), (size_t)dom.numElem()))) return st;
    if ((st = lg_set_scalar(g, "time", dom.time())) ||
        (st = lg_set_scalar(g, "deltatime", dom.deltatime())) ||
        (st = lg_set_scalar(g, "dtcourant", dom.dtcourant())) ||
        (st = lg_set_scalar(g, "dthydro", dom.dthydro())) ||
        (st = lg_set_scalar(g, "cycle", dom.cycle())))
        return st;

    const int run = lg_step(g, n);
    if (run > 0) return run;

    for (const FieldBinding &f : kNodeFields)
        if ((st = lg_get_field(g, f.name, &(dom.*f.get)(0), (size_t)dom.numNode()))) return st;
    for (const FieldBinding &f : kElemFields)
        if ((st = lg_get_field(g, f.name, &(dom.*f.get)(0), (size_t)dom.numElem()))) return st;
    double v;
    if ((st = lg_get_scalar(g, "time", &v))) return st;
    dom.time() = v;
    if ((st = lg_get_scalar(g, "deltatime", &v))) return st;
    dom.deltatime() = v;
    if ((st = lg_get_scalar(g, "dtcourant", &v))) return st;
    dom.dtcourant() = v;
    if ((st = lg_get_scalar(g, "dthydro", &v))) return st;
    dom.dthydro() = v;
    if ((st = lg_get_scalar(g, "cycle", &v))) return st;
    dom.cycle() = (Int_t)v;
    return run;
}
