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
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
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
    printf("\n\n");
}

[[noreturn]] void parse_error(const char *msg)
{
    printf("%s\n", msg);
    exit(-1);
}

}  // namespace

int main(int argc, char *argv[])
{
    lg_opts o;
    lg_default_opts(&o);
    int showProg = 0, quiet = 0, numFiles = (1 + 10) / 9;
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
    lg_destroy(d);
    return 0;
}
