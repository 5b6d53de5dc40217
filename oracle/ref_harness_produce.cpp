/*
 * Reference harness (test infrastructure only): compiles the reference CPU
 * production program produce.cpp from its own source (found through -I on
 * the reference checkout) inside a namespace, and exports its routines with
 * C linkage so the tests can call them beside the oracle.  Nothing of the
 * reference is copied here.
 */
#include <iostream>
#include <sstream>
#include <cstdlib>
#include <cstdio>
#include <cstdint>
#include <cmath>
#include <vector>
#include <limits>
#include <fstream>
#include <iomanip>
#include <ctime>
#include <algorithm>
#include <getopt.h>
#include <mpi.h>
#include "Random123/philox.h"
#include "Random123/examples/uniform.hpp"

namespace ref_produce {
#define main ref_main
#include "produce.cpp"
#undef main
}

extern "C" {
/* produce.cpp:421-511; lattice int[N]; naver/index built as produce.cpp:76-93 */
void refp_mcs(unsigned L, unsigned worker, int *lattice, unsigned long *hist, double *log_weight,
              int *E_Delta, int *energy, int *mag, unsigned iter, unsigned seed,
              unsigned long long therm, unsigned long long nup, const int *index, const int *naver)
{
    ref_produce::L = L;
    ref_produce::N = L * L;
    ref_produce::mcs(lattice, 2.0, 0.0, hist, const_cast<int *>(index), const_cast<int *>(naver), nullptr,
                     log_weight, E_Delta, energy, worker, mag, iter, seed, therm, nup);
}
void refp_observables(double beta, double delta, unsigned N, unsigned long *h, double *boltz, double *lnw,
                      double *M_jacks, double *sus_jacks, unsigned k)
{
    ref_produce::N = N;
    ref_produce::observables(beta, delta, N, h, boltz, lnw, M_jacks, sus_jacks, k);
}
void refp_jakknife(double *M, double *avg, double *err, int J, unsigned range)
{
    ref_produce::jakknife(M, avg, err, J, range);
}
void refp_weight_shift(double beta, double delta, unsigned N, double *lnw)
{
    ref_produce::N = N;
    ref_produce::weight_shift(beta, delta, lnw);
}
int refp_total_energy(unsigned L, int *lattice)
{
    ref_produce::L = L;
    ref_produce::N = L * L;
    return ref_produce::total_energy(lattice);
}
int refp_main(int argc, char **argv) { return ref_produce::ref_main(argc, argv); }
}
