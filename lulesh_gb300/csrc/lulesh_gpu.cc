// lulesh_gpu.cc -- drop-in command line for the reference executable.
//
// Accepts the reference options (-q -i -s -r -b -c -f -p -v -h, parsed with
// the same rules as ParseCommandLineOptions, lulesh-util.cc:63-171), prints
// the same banner (lulesh.cc:2694-2708), per-cycle progress line
// (lulesh.cc:2750-2756) and end-of-run report (lulesh-util.cc:175-230), and
// exits with the reference's codes: -1 VolumeError, -2 QStopError.
// Additional long options choose the device path:
//   --precision fp64|fp64-fma|mixed   (default fp64)
//   --device N
// and write the final state for visualisation without Silo (which -v needs,
// as in the reference):
//   --viz-vtk FILE   the fields of the reference's viz dump (lulesh-viz.cc:
//                    mesh, regions, e, p, v, q, speed, xd, yd, zd) as a binary
//                    legacy VTK unstructured grid
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>
#include <vector>

#include "lulesh_gb300.h"

namespace {

// StrToInt, lulesh-util.cc:13-29: strtol, accepted when the token is
// non-empty and ends at a blank or the end of the string
bool str_to_int(const char *token, int *out)
{
    if (!token) return false;
    char *end = nullptr;
    const long v = strtol(token, &end, 10);
    *out = (int)v;
    return end != token && (*end == ' ' || *end == '\0');
}

void usage(const char *exe)
{
    printf("Usage: %s [opts]\n", exe);
    printf(" where [opts] is one or more of:\n");
    printf(" -q              : quiet mode - suppress all stdout\n");
    printf(" -i <iterations> : number of cycles to run\n");
    printf(" -s <size>       : length of cube mesh along side\n");
    printf(" -r <numregions> : Number of distinct regions (def: 11)\n");
    printf(" -b <balance>    : Load balance between regions of a domain (def: 1)\n");
    printf(" -c <cost>       : Extra cost of more expensive regions (def: 1)\n");
    printf(" -f <numfiles>   : Number of files to split viz dump into (def: (np+10)/9)\n");
    printf(" -p              : Print out progress\n");
    printf(" -v              : Output viz file (requires compiling with -DVIZ_MESH\n");
    printf(" -h              : This message\n");
    printf(" --precision <fp64|fp64-fma|mixed> : device arithmetic (def: fp64)\n");
    printf(" --device <n>    : CUDA device ordinal (def: 0)\n");
    printf(" --viz-vtk <file>: write the final mesh and fields as legacy VTK\n");
    printf("\n\n");
}

[[noreturn]] void parse_error(const char *msg)
{
    printf("%s\n", msg);
    exit(-1);
}

// legacy VTK binary data is big-endian
template <typename T>
void put_be(FILE *f, const std::vector<T> &v)
{
    std::vector<unsigned char> b(v.size() * sizeof(T));
    for (size_t i = 0; i < v.size(); ++i) {
        unsigned char w[sizeof(T)];
        memcpy(w, &v[i], sizeof(T));
        for (size_t k = 0; k < sizeof(T); ++k) b[i * sizeof(T) + k] = w[sizeof(T) - 1 - k];
    }
    fwrite(b.data(), 1, b.size(), f);
}

std::vector<double> get_f64(lg_domain *d, const char *name, size_t n)
{
    std::vector<double> v(n);
    lg_get_field(d, name, v.data(), n);
    return v;
}

std::vector<float> get_f32(lg_domain *d, const char *name, size_t n)
{
    const std::vector<double> v = get_f64(d, name, n);
    return std::vector<float>(v.begin(), v.end());
}

// The content of DumpDomainToVisit (lulesh-viz.cc:120-259) in a binary legacy
// VTK file: the cycle and time (:159-160), node coordinates in single
// precision (:150-165), the hexahedra (:131-146), each element's region number
// (:171-179), e, p, v, q per element (:181-218) and speed, xd, yd, zd per node
// (:220-252), all values in single precision as the reference writes them.
// LULESH's corner order is VTK's hexahedron order.
int write_vtk(lg_domain *d, const char *path)
{
    double ne, nn, cyc, time;
    lg_get_scalar(d, "numElem", &ne);
    lg_get_scalar(d, "numNode", &nn);
    lg_get_scalar(d, "cycle", &cyc);
    lg_get_scalar(d, "time", &time);
    const size_t E = (size_t)ne, N = (size_t)nn;
    FILE *f = fopen(path, "wb");
    if (!f) return -1;
    fprintf(f, "# vtk DataFile Version 3.0\nLULESH cycle %d time %.9e\nBINARY\n"
               "DATASET UNSTRUCTURED_GRID\nPOINTS %zu float\n", (int)cyc, time, N);
    const std::vector<float> x = get_f32(d, "x", N), y = get_f32(d, "y", N),
                             z = get_f32(d, "z", N);
    std::vector<float> xyz(3 * N);
    for (size_t i = 0; i < N; ++i) {
        xyz[3 * i] = x[i];
        xyz[3 * i + 1] = y[i];
        xyz[3 * i + 2] = z[i];
    }
    put_be(f, xyz);
    std::vector<int32_t> nl(8 * E);
    lg_get_field(d, "nodelist", nl.data(), nl.size());
    std::vector<int32_t> cells(9 * E);
    for (size_t e = 0; e < E; ++e) {
        cells[9 * e] = 8;
        for (int j = 0; j < 8; ++j) cells[9 * e + 1 + j] = nl[8 * e + j];
    }
    fprintf(f, "\nCELLS %zu %zu\n", E, 9 * E);
    put_be(f, cells);
    fprintf(f, "\nCELL_TYPES %zu\n", E);
    put_be(f, std::vector<int32_t>(E, 12));  // VTK_HEXAHEDRON
    fprintf(f, "\nCELL_DATA %zu\nSCALARS regions int 1\nLOOKUP_TABLE default\n", E);
    std::vector<int32_t> reg(E);
    lg_get_field(d, "regNumList", reg.data(), E);
    put_be(f, reg);
    for (const char *name : {"e", "p", "v", "q"}) {
        fprintf(f, "\nSCALARS %s float 1\nLOOKUP_TABLE default\n", name);
        put_be(f, get_f32(d, name, E));
    }
    const std::vector<float> fx = get_f32(d, "xd", N), fy = get_f32(d, "yd", N),
                             fz = get_f32(d, "zd", N);
    std::vector<float> speed(N);
    for (size_t i = 0; i < N; ++i)
        speed[i] = float(std::sqrt((fx[i] * fx[i]) + (fy[i] * fy[i]) + (fz[i] * fz[i])));
    fprintf(f, "\nPOINT_DATA %zu\n", N);
    const std::pair<const char *, const std::vector<float> *> nodal[4] = {
        {"speed", &speed}, {"xd", &fx}, {"yd", &fy}, {"zd", &fz}};
    for (auto &v : nodal) {
        fprintf(f, "SCALARS %s float 1\nLOOKUP_TABLE default\n", v.first);
        put_be(f, *v.second);
        fprintf(f, "\n");
    }
    return fclose(f) == 0 ? 0 : -1;
}

}  // namespace

int main(int argc, char *argv[])
{
    lg_opts o;
    lg_default_opts(&o);
    int showProg = 0, quiet = 0, numFiles = (1 + 10) / 9;
    const char *vtkPath = nullptr;
    (void)numFiles;
    for (int i = 1; i < argc;) {
        const char *a = argv[i];
        auto int_arg = [&](int *dst, const char *missing, const char *bad) {
            if (i + 1 >= argc) parse_error(missing);
            if (!str_to_int(argv[i + 1], dst)) parse_error(bad);
            i += 2;
        };
        if (!strcmp(a, "-i"))
            int_arg(&o.its, "Missing integer argument to -i",
                    "Parse Error on option -i integer value required after argument\n");
        else if (!strcmp(a, "-s"))
            int_arg(&o.nx, "Missing integer argument to -s\n",
                    "Parse Error on option -s integer value required after argument\n");
        else if (!strcmp(a, "-r"))
            int_arg(&o.numReg, "Missing integer argument to -r\n",
                    "Parse Error on option -r integer value required after argument\n");
        else if (!strcmp(a, "-f"))
            int_arg(&numFiles, "Missing integer argument to -f\n",
                    "Parse Error on option -f integer value required after argument\n");
        else if (!strcmp(a, "-b"))
            int_arg(&o.balance, "Missing integer argument to -b\n",
                    "Parse Error on option -b integer value required after argument\n");
        else if (!strcmp(a, "-c"))
            int_arg(&o.cost, "Missing integer argument to -c\n",
                    "Parse Error on option -c integer value required after argument\n");
        else if (!strcmp(a, "-p")) {
            showProg = 1;
            i++;
        } else if (!strcmp(a, "-q")) {
            quiet = 1;
            i++;
        } else if (!strcmp(a, "-v")) {
            parse_error("Use of -v requires compiling with -DVIZ_MESH\n");
        } else if (!strcmp(a, "-h")) {
            usage(argv[0]);
            exit(0);
        } else if (!strcmp(a, "--device")) {
            int_arg(&o.device, "Missing integer argument to --device",
                    "Parse Error on option --device integer value required after argument\n");
        } else if (!strcmp(a, "--viz-vtk")) {
            if (i + 1 >= argc) parse_error("Missing argument to --viz-vtk");
            vtkPath = argv[i + 1];
            i += 2;
        } else if (!strcmp(a, "--precision")) {
            if (i + 1 >= argc) parse_error("Missing argument to --precision");
            const char *p = argv[i + 1];
            if (!strcmp(p, "fp64"))
                o.precision = LG_FP64;
            else if (!strcmp(p, "fp64-fma"))
                o.precision = LG_FP64_FMA;
            else if (!strcmp(p, "mixed"))
                o.precision = LG_MIXED;
            else
                parse_error("Parse Error on option --precision: fp64, fp64-fma or mixed");
            i += 2;
        } else {
            char msg[80];
            usage(argv[0]);
            snprintf(msg, sizeof(msg), "ERROR: Unknown command line argument: %s\n", a);
            parse_error(msg);
        }
    }

    if (!quiet) {
        std::cout << "Running problem size " << o.nx << "^3 per domain until completion\n";
        std::cout << "Num processors: " << 1 << "\n";
        std::cout << "Total number of elements: " << ((long long)o.nx * o.nx * o.nx) << " \n\n";
        std::cout << "To run other sizes, use -s <integer>.\n";
        std::cout << "To run a fixed number of iterations, use -i <integer>.\n";
        std::cout << "To run a more or less balanced region set, use -b <integer>.\n";
        std::cout << "To change the relative costs of regions, use -c <integer>.\n";
        std::cout << "To print out progress, use -p\n";
        std::cout << "To write an output file for VisIt, use -v\n";
        std::cout << "See help (-h) for more options\n\n";
    }

    lg_domain *d = nullptr;
    int st = lg_create(&o, &d);
    if (st) {
        fprintf(stderr, "lulesh_gpu: %s\n", lg_last_error());
        return st > 0 ? st : st;
    }
    const auto t0 = std::chrono::steady_clock::now();
    if (showProg && !quiet) {
        // one synchronised cycle at a time, as the reference prints each one
        for (;;) {
            double time, stop, cyc, dt;
            lg_get_scalar(d, "time", &time);
            lg_get_scalar(d, "stoptime", &stop);
            lg_get_scalar(d, "cycle", &cyc);
            if (!(time < stop && cyc < o.its)) break;
            st = lg_step(d, 1);
            if (st) break;
            lg_get_scalar(d, "cycle", &cyc);
            lg_get_scalar(d, "time", &time);
            lg_get_scalar(d, "deltatime", &dt);
            std::cout << "cycle = " << (int)cyc << ", " << std::scientific << "time = " << time
                      << ", " << "dt=" << dt << "\n";
            std::cout.unsetf(std::ios_base::floatfield);
        }
    } else {
        st = lg_run(d);
    }
    const double elapsed =
        std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (st > 0) {
        fprintf(stderr, "lulesh_gpu: %s\n", lg_last_error());
        lg_destroy(d);
        return st;
    }
    if (st < 0) {
        lg_destroy(d);
        exit(st);  // VolumeError / QStopError, as the reference
    }
    if (!quiet) {
        std::vector<char> buf(4096);
        lg_report(d, elapsed, buf.data(), buf.size());
        std::cout << buf.data();
    }
    if (vtkPath && write_vtk(d, vtkPath) != 0) {
        printf("Error writing out viz file %s\n", vtkPath);
        lg_destroy(d);
        return 1;
    }
    lg_destroy(d);
    return 0;
}
