/*
 * Reference harness (test infrastructure only): compiles the reference CPU
 * weight program muca_mag.cpp from its own source inside a namespace and
 * exports its routines with C linkage for the tests.
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
#include <getopt.h>
#include <mpi.h>
#include "Random123/philox.h"
#include "Random123/examples/uniform.hpp"

namespace ref_mucamag {
#define main ref_main
#include "muca_mag.cpp"
#undef main
}

extern "C" {
/* muca_mag.cpp:312-393 */
void refm_mcs(unsigned L, unsigned worker, int *lattice, unsigned long long *hist, double *log_weight,
              const int *index, const int *naver, int *energy, int *E_delta, unsigned iter, unsigned seed,
              unsigned long long therm, unsigned long long nup)
{
    ref_mucamag::L = L;
    ref_mucamag::N = L * L;
    ref_mucamag::mcs(lattice, hist, log_weight, const_cast<int *>(index), const_cast<int *>(naver), energy,
                     E_delta, worker, iter, seed, therm, nup);
}
void refm_hist_range(unsigned N, unsigned long long *h, int *start, int *end)
{
    ref_mucamag::N = N;
    ref_mucamag::hist_range(h, *start, *end);
}
double refm_kull_leiber(unsigned N, unsigned long long *h)
{
    ref_mucamag::N = N;
    return ref_mucamag::kull_leiber(h);
}
void refm_weight_recursion(unsigned N, unsigned long long *h, double *p_acc, int start, int end, double *lnw)
{
    ref_mucamag::N = N;
    ref_mucamag::weight_recursion(h, p_acc, start, end, lnw);
}
}
