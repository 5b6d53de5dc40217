/*
 * Reference harness (test infrastructure only): compiles the reference GPU
 * programs muca_delta_multigpu.cu and produce2_multigpu.cu from their own
 * sources inside namespaces and exports their HOST routines (histogram
 * range, Kullback-Leibler divergence, weight recursion, jackknife, weight
 * shift, observables) with C linkage, so the tests can call them on a
 * machine without a GPU.  No kernel of theirs is launched from here.
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
#include <errno.h>
#include "Random123/philox.h"
#include "Random123/examples/uniform.hpp"

namespace ref_wgpu {
#define main ref_main
#include "muca_delta_multigpu.cu"
#undef main
}
namespace ref_pgpu {
#define main ref_main
#include "produce2_multigpu.cu"
#undef main
}

extern "C" {
void refg_hist_range(unsigned long long *h, int N, int *start, int *end) { ref_wgpu::hist_range(h, N, *start, *end); }
double refg_kull_leibler(unsigned long long *h, int N) { return ref_wgpu::kull_leibler(h, N); }
void refg_weight_recursion(unsigned N, unsigned long long *h, double *p_acc, int s, int e, double *lnw)
{
    ref_wgpu::weight_recursion(N, h, p_acc, s, e, lnw);
}
void refg_jakknife(double *M, double *avg, double *err, unsigned J) { ref_wgpu::jakknife(M, avg, err, J); }
void refg_weight_shift(double beta, double delta, unsigned N, double *lnw) { ref_pgpu::weight_shift(beta, delta, N, lnw); }
void refg_observables(double beta, double delta, unsigned N, unsigned long long *h, double *boltz, double *lnw,
                      double *M_jacks, double *sus_jacks, unsigned k)
{
    ref_pgpu::observables(beta, delta, N, h, boltz, lnw, M_jacks, sus_jacks, k);
}
void refg_jakknife_range(double *M, double *avg, double *err, int J, unsigned range)
{
    ref_pgpu::jakknife(M, avg, err, J, range);
}
}
