// produce_gpu -- drop-in replacement for the reference program of the same
// name (produce2_multigpu.cu, main at :91-363) on one GB300.
//
//   produce_gpu L first_gpu last_gpu range jacks therm_mult nup_mult delta gap
//               [--device=D] [--chains=NW] [--jack-blocks] [--binder] [--kernel=0..3]
//
// Reads ./fss/L<L>/weight_mpi_T050c16_M200_JACK0_DKL1e-4.txt (:205-226), runs
// for each of `range` Delta points a thermalisation launch and a production
// launch per device (:293-312), reweights each device's (E_Delta, M)
// histogram (:318, :498-518), jackknifes over the devices (:320-321) and
// writes ./fss/L<L>/observables_gpu... (:350-358).  The first_gpu..last_gpu
// range becomes that many emulated devices on one GPU, each with its own
// histogram and the reference's per-device seeds.
//
// Options of this project:
//   --jack-blocks  jackknife over `jacks` production blocks per Delta point
//                  (each block its own histogram, summed over devices, seeds
//                  of the block loop the reference left commented out,
//                  :324-347) instead of over devices; with one device the
//                  reference's error column is NaN, with blocks it is not;
//   --binder       also writes the Binder cumulant U4 = 1 - <M^4>/(3<M^2>^2)
//                  per Delta point to observables_binder_gpu...;
//   --reuse-histogram  one thermalisation and one production run (with the
//                  first Delta point's seeds) serve every Delta point.  The
//                  sweep's weights are the file's at every point (the shift
//                  only enters the reweighting), so the simulation does not
//                  depend on Delta and each point only reweights the same
//                  histogram(s) with its own shifted weights: `range` times
//                  fewer sweeps.  The first line equals the one without the
//                  option;
//   --load-chains=FILE  start the chains from a chain file written by
//                  multigpu_weight --save-chains (the weight run's final
//                  lattices, spread over E_Delta by the converged walk)
//                  instead of fresh random spins (:126-140);
//   ./fss/L<L> is created when missing.
#include <fstream>
#include <iomanip>
#include <iostream>
#include <sstream>

#include "cli_common.h"

int main(int argc, char **argv)
{
    std::vector<std::string> pos;
    cli::Options opt;
    cli::parse(argc, argv, pos, opt);
    if (pos.size() < 9) {
        std::fprintf(stderr,
                     "usage: %s L first_gpu last_gpu range jacks therm_mult nup_mult delta gap\n"
                     "          [--device=D] [--chains=NW] [--jack-blocks] [--binder] [--reuse-histogram]\n"
                     "          [--kernel=0..3] [--load-chains=FILE]\n",
                     argv[0]);
        return 2;
    }
    const std::string Ls = pos[0];
    const unsigned L = (unsigned)std::stoi(pos[0]);
    const int first_gpu = std::atoi(pos[1].c_str()), last_gpu = std::atoi(pos[2].c_str());
    const unsigned NofGPU = (unsigned)(1 + last_gpu - first_gpu);
    const unsigned range = (unsigned)std::stoi(pos[3]);
    const unsigned JACKS = (unsigned)std::stoi(pos[4]);
    double delta = std::atof(pos[7].c_str()), beta = 1.0 / 0.5;
    const double delta_i = delta, gap = std::atof(pos[8].c_str());
    if (last_gpu < first_gpu || L < 2 || range == 0) {
        std::fprintf(stderr, "error: invalid arguments\n");
        return 2;
    }
    const bool blocks = opt.has("jack-blocks") && JACKS > 0;
    const bool reuse = opt.has("reuse-histogram");
    const unsigned N = L * L;
    // weight file: "i lnW" pairs (:205-226), checked before any device work
    std::vector<double> log_weight;
    {
        std::string why;
        if (!cli::read_weight_pairs("./fss/L" + Ls + "/weight_mpi_T050c16_M200_JACK0_DKL1e-4.txt", N, log_weight,
                                    why))
            cli::die_io(why);
    }
    const int device = (int)opt.num("device", first_gpu);
    uint32_t NUM_WORKERS = 0;
    if (opt.has("chains")) {
        NUM_WORKERS = (uint32_t)opt.num("chains", 0);
    } else if (muca_default_chains(device, &NUM_WORKERS) != MUCA_OK) {
        cli::die("device query", nullptr);
    }
    // --load-chains: start every device's chains from a weight run's final
    // lattices (device g takes chains g*NW .. g*NW + NW - 1), checked before
    // any device work
    std::vector<int8_t> start_lat;
    if (opt.has("load-chains")) {
        std::string why;
        if (!cli::read_chains(opt.str("load-chains", ""), L, NUM_WORKERS * NofGPU, start_lat, why))
            cli::die_chains(why);
    }

    // one context per emulated device: each has its own 2D histogram
    std::vector<muca_ctx *> ctx(NofGPU, nullptr);
    for (unsigned g = 0; g < NofGPU; ++g) {
        muca_params prm{};
        prm.L = L;
        prm.nchains = NUM_WORKERS;
        prm.ndev = 1;
        prm.dev_offset = g;
        prm.device = device;
        prm.rounds = 7;
        prm.mode = MUCA_MODE_PRODUCE;
        prm.kernel = (uint32_t)opt.num("kernel", 0);
        if (muca_create(&prm, &ctx[g]) != MUCA_OK) cli::die("create", nullptr);
        if (muca_init_chains(ctx[g], MUCA_INIT_PRODUCE, 0) != MUCA_OK) cli::die("init chains", ctx[g]);
        if (!start_lat.empty() &&
            muca_set_lattice(ctx[g], start_lat.data() + (size_t)g * NUM_WORKERS * N, (size_t)NUM_WORKERS * N) != MUCA_OK)
            cli::die("set lattice", ctx[g]);
    }
    cli::ensure_dir("./fss/L" + Ls);

    for (unsigned g = 0; g < NofGPU; ++g)
        if (muca_set_weights(ctx[g], log_weight.data(), N + 1) != MUCA_OK) cli::die("set weights", ctx[g]);

    const unsigned long long therm_run = (unsigned long long)N * std::atoi(pos[5].c_str());
    const unsigned long long NUPDATES = (unsigned long long)N * std::atoi(pos[6].c_str());
    std::cout << "\n TOTAL UPDATES : " << NUPDATES * NUM_WORKERS << " updates by each core : " << NUPDATES
              << " Therm run : " << therm_run << std::endl;

    std::vector<double> avg_M(range), error_M(range), avg_sus(range), error_sus(range), avg_u4(range),
        error_u4(range);
    const unsigned nj = blocks ? JACKS : NofGPU;
    if (reuse) {
        // [l][unit]: the jackknife quantities of every Delta point
        std::vector<double> Mq((size_t)range * nj), Sq((size_t)range * nj), Uq((size_t)range * nj);
        std::vector<double> sums((size_t)range * nj * 4, 0.0);
        // reweights the device's current histogram at every Delta point, with
        // the reweighting weights shifted from the file's exactly as the loop
        // below shifts them point by point
        auto scan_deltas = [&](unsigned unit, unsigned g) {
            if (muca_set_weights(ctx[g], log_weight.data(), N + 1) != MUCA_OK) cli::die("set weights", ctx[g]);
            double d = delta_i;
            for (unsigned l = 0; l < range; ++l) {
                d = d + gap / (double)range;
                if (muca_weight_shift(ctx[g], beta, d) != MUCA_OK) cli::die("weight shift", ctx[g]);
                muca_observables o{};
                if (muca_compute_observables(ctx[g], beta, d, &o) != MUCA_OK) cli::die("observables", ctx[g]);
                const size_t k = (size_t)l * nj + unit;
                Mq[k] = o.m_abs;
                Sq[k] = o.chi;
                Uq[k] = o.u4;
                sums[4 * k] += o.sum;
                sums[4 * k + 1] += o.m1;
                sums[4 * k + 2] += o.m2;
                sums[4 * k + 3] += o.m4;
            }
        };
        // the first Delta point's thermalisation and production seeds (l = 0)
        for (unsigned g = 0; g < NofGPU; ++g)
            if (muca_sweep(ctx[g], 0, 100u, 1000u, therm_run, 0) != MUCA_OK) cli::die("sweep", ctx[g]);
        if (!blocks) {
            for (unsigned g = 0; g < NofGPU; ++g)
                if (muca_sweep(ctx[g], 0, 100u, 2000u, 0, NUPDATES) != MUCA_OK) cli::die("sweep", ctx[g]);
            for (unsigned g = 0; g < NofGPU; ++g) scan_deltas(g, g);
        } else {
            for (unsigned jj = 0; jj < JACKS; ++jj)
                for (unsigned g = 0; g < NofGPU; ++g) {
                    if (muca_sweep(ctx[g], jj, 100u, 2000u, 0, NUPDATES) != MUCA_OK) cli::die("sweep", ctx[g]);
                    scan_deltas(jj, g);
                }
            for (size_t k = 0; k < (size_t)range * nj; ++k) {
                const double s = sums[4 * k], m1 = sums[4 * k + 1], m2 = sums[4 * k + 2], m4 = sums[4 * k + 3];
                Mq[k] = m1 / s;
                Sq[k] = (m2 / s - (m1 / s) * (m1 / s)) * beta / (double)N;
                Uq[k] = 1.0 - (m4 / s) / (3.0 * (m2 / s) * (m2 / s));
            }
        }
        for (unsigned l = 0; l < range; l++) {
            const size_t k = (size_t)l * nj;
            muca_jackknife(ctx[0], &Mq[k], nj, &avg_M[l], &error_M[l]);
            muca_jackknife(ctx[0], &Sq[k], nj, &avg_sus[l], &error_sus[l]);
            muca_jackknife(ctx[0], &Uq[k], nj, &avg_u4[l], &error_u4[l]);
        }
    }
    for (unsigned l = 0; l < range && !reuse; l++) {
        std::cout << "L" << Ls << " Progress...  " << 100 * l / range << "%" << "\r" << std::flush;
        delta = delta + gap / (double)range;
        for (unsigned g = 0; g < NofGPU; ++g) {
            if (muca_weight_shift(ctx[g], beta, delta) != MUCA_OK) cli::die("weight shift", ctx[g]);
            // thermalisation launch: iter 0, seed SEED+1000*GPU+l (:301)
            if (muca_sweep(ctx[g], 0, 100u + l, 1000u, therm_run, 0) != MUCA_OK) cli::die("sweep", ctx[g]);
        }
        std::vector<double> M_jacks(nj, 0.0), sus_jacks(nj, 0.0), u4_jacks(nj, 0.0);
        if (!blocks) {
            for (unsigned g = 0; g < NofGPU; ++g) {
                // production launch: iter l, seed SEED+2000*GPU (:311)
                if (muca_sweep(ctx[g], l, 100u, 2000u, 0, NUPDATES) != MUCA_OK) cli::die("sweep", ctx[g]);
            }
            for (unsigned g = 0; g < NofGPU; ++g) {
                muca_observables o{};
                if (muca_compute_observables(ctx[g], beta, delta, &o) != MUCA_OK) cli::die("observables", ctx[g]);
                M_jacks[g] = o.m_abs;
                sus_jacks[g] = o.chi;
                u4_jacks[g] = o.u4;
            }
        } else {
            for (unsigned jj = 0; jj < JACKS; ++jj) {
                double s = 0, m1 = 0, m2 = 0, m4 = 0;
                for (unsigned g = 0; g < NofGPU; ++g) {
                    // block jj: iter jj, seed SEED+2000*GPU+l (:332)
                    if (muca_sweep(ctx[g], jj, 100u + l, 2000u, 0, NUPDATES) != MUCA_OK) cli::die("sweep", ctx[g]);
                    muca_observables o{};
                    if (muca_compute_observables(ctx[g], beta, delta, &o) != MUCA_OK) cli::die("observables", ctx[g]);
                    s += o.sum;
                    m1 += o.m1;
                    m2 += o.m2;
                    m4 += o.m4;
                }
                M_jacks[jj] = m1 / s;
                sus_jacks[jj] = (m2 / s - (m1 / s) * (m1 / s)) * beta / (double)N;
                u4_jacks[jj] = 1.0 - (m4 / s) / (3.0 * (m2 / s) * (m2 / s));
            }
        }
        muca_jackknife(ctx[0], M_jacks.data(), nj, &avg_M[l], &error_M[l]);
        muca_jackknife(ctx[0], sus_jacks.data(), nj, &avg_sus[l], &error_sus[l]);
        muca_jackknife(ctx[0], u4_jacks.data(), nj, &avg_u4[l], &error_u4[l]);
    }

    std::ofstream producefile;
    std::stringstream pdname;
    pdname << "./fss/L" << Ls << "/observables_gpu" << NofGPU << "_T050_JACKgpu_THERM" << pos[5] << "N_NUP" << pos[6]
           << "N_delta" << pos[7] << "to" << pos[8] << "noreset.txt";
    producefile.open(pdname.str().c_str());
    for (size_t i = 0; i < range; i++) {
        producefile << delta_i + gap * (i + 1) / (double)range << " " << std::setprecision(10) << avg_M[i] << " "
                    << std::setprecision(10) << error_M[i] << " " << std::setprecision(10) << avg_sus[i] << " "
                    << std::setprecision(10) << error_sus[i] << std::endl;
    }
    producefile.close();
    if (opt.has("binder")) {
        std::ofstream bf(("./fss/L" + Ls + "/observables_binder_gpu" + std::to_string(NofGPU) + "_T050_THERM" + pos[5] +
                          "N_NUP" + pos[6] + "N_delta" + pos[7] + "to" + pos[8] + ".txt").c_str());
        bf << "#delta U4_avg U4_err" << std::endl;
        for (size_t i = 0; i < range; i++)
            bf << delta_i + gap * (i + 1) / (double)range << " " << std::setprecision(10) << avg_u4[i] << " "
               << error_u4[i] << std::endl;
    }
    for (muca_ctx *c : ctx) muca_destroy(c);
    return 0;
}
