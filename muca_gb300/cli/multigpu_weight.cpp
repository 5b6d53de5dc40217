// multigpu_weight -- drop-in replacement for the reference program of the same
// name (muca_delta_multigpu.cu, main at :87-546) on one GB300.
//
//   multigpu_weight L starting_gpu last_gpu jacks starting_M recursive_update continuing [rand_config]
//                   [--device=D] [--chains=NW] [--max-iter=K] [--flat=minmean] [--kernel=0..3]
//
// Same positional command line (weight.bash:15), same stdout banners and the
// same files under ./fss/L<L>/: shortiter_gpu... (one line per iteration,
// :367-370,439), weight_gpu... (on convergence, :485-493) and
// converge_result_gpu... (:509-524).  The starting_gpu..last_gpu range becomes
// last_gpu-starting_gpu+1 emulated devices on device starting_gpu (or
// --device), each with the reference's per-device seeds.
//
// Deliberate differences, each a documented fix of the reference:
//   * recursive_update=1 applies weight_recursion (the reference parses the
//     flag but never calls the routine, :468);
//   * rand_config=0 starts every spin at +1 (the reference never reads it);
//   * total_run is accumulated in 64 bits (the reference multiplies in 32);
//   * --max-iter bounds the otherwise endless iteration loop (:374);
//   * ./fss/L<L> is created when missing (the reference writes nothing then).
#include <fstream>
#include <iomanip>
#include <iostream>
#include <sstream>

#include "cli_common.h"

namespace {

struct JackLog {
    std::ofstream *out;
    double total_kernel_ms = 0;
    double nwidth_time_s = 0;
    uint64_t nwidth_step = 0;
    bool reach = false;
    uint32_t N = 0, width = 0;
};

void on_iter(const muca_iter_record *r, void *user)
{
    JackLog &j = *static_cast<JackLog *>(user);
    j.total_kernel_ms += r->kernel_ms;
    j.width = r->width;
    // "#iter width D_KL mcs_time memcpy_time accumulated_time NUPDATES acc_NUP" (:439)
    if (j.out && j.out->is_open())
        *j.out << r->k << " " << r->width_temp << " " << r->d_kl << " " << (float)r->kernel_ms * 1e-3 << " "
               << (float)r->memcpy_ms * 1e-3 << " " << j.total_kernel_ms * 1e-3 << " " << r->nupdates << " "
               << r->total_run << std::endl;
    if (r->width == j.N && !j.reach) {  // :441-446
        std::cout << "Width reached N... Total mcs time : " << j.total_kernel_ms * 1e-3 << std::endl;
        j.nwidth_time_s = j.total_kernel_ms * 1e-3;
        j.nwidth_step = r->total_run;
        j.reach = true;
    }
}

}  // namespace

int main(int argc, char **argv)
{
    std::vector<std::string> pos;
    cli::Options opt;
    cli::parse(argc, argv, pos, opt);
    if (pos.size() < 7) {
        std::fprintf(stderr,
                     "usage: %s L starting_gpu last_gpu jacks starting_M recursive_update continuing [rand_config]\n"
                     "          [--device=D] [--chains=NW] [--max-iter=K] [--flat=minmean] [--kernel=0..3]\n"
                     "          [--save-chains=FILE] [--hist-dump]\n",
                     argv[0]);
        return 2;
    }
    const std::string Ls = pos[0];
    const unsigned L = (unsigned)std::atoi(pos[0].c_str());
    const int starting_gpu = std::atoi(pos[1].c_str()), last_gpu = std::atoi(pos[2].c_str());
    const unsigned jacks = (unsigned)std::atoi(pos[3].c_str());
    const unsigned initNUPDATES = (unsigned)std::atoi(pos[4].c_str());
    const bool recursion = std::atoi(pos[5].c_str()) != 0;
    const int extrapolation = std::atoi(pos[6].c_str()) != 0;
    const int rand_config = pos.size() > 7 ? std::atoi(pos[7].c_str()) : 1;
    const unsigned NofGPU = (unsigned)(1 + last_gpu - starting_gpu);
    if (last_gpu < starting_gpu || L < 2 || jacks == 0 || initNUPDATES == 0) {
        std::fprintf(stderr, "error: invalid arguments\n");
        return 2;
    }
    const unsigned N = L * L;
    std::vector<double> log_weight((size_t)N + 1, 0.0);
    if (extrapolation) {  // :223-235, one value per line; checked before any device work
        std::string why;
        if (!cli::read_weight_column("./fss/L" + Ls + "/initweight_L128_T050.txt", N, log_weight, why))
            cli::die_io(why);
    }
    const int device = (int)opt.num("device", starting_gpu);
    uint32_t NUM_WORKERS = 0;
    if (opt.has("chains")) {
        NUM_WORKERS = (uint32_t)opt.num("chains", 0);
    } else if (muca_default_chains(device, &NUM_WORKERS) != MUCA_OK) {
        cli::die("device query", nullptr);
    }
    if (NofGPU > 1)
        std::fprintf(stderr, "note: devices %d..%d run as %u emulated devices on device %d\n", starting_gpu, last_gpu,
                     NofGPU, device);

    muca_params prm{};
    prm.L = L;
    prm.nchains = NUM_WORKERS;
    prm.ndev = NofGPU;
    prm.device = device;
    prm.rounds = 7;
    prm.mode = MUCA_MODE_WEIGHT;
    prm.kernel = (uint32_t)opt.num("kernel", 0);
    muca_ctx *ctx = nullptr;
    if (muca_create(&prm, &ctx) != MUCA_OK) cli::die("create", nullptr);
    cli::ensure_dir("./fss/L" + Ls);

    if (muca_set_weights(ctx, log_weight.data(), N + 1) != MUCA_OK) cli::die("set weights", ctx);

    const unsigned therm_coeff = 1;
    unsigned width = 10;
    std::vector<double> total_kernel(jacks, 0), total_mem(jacks, 0), Nwidth_time(jacks, 0);
    std::vector<double> total_run_d(jacks, 0), Nwidth_step_d(jacks, 0);
    std::vector<uint64_t> total_run(jacks, 0), Nwidth_step(jacks, 0);
    std::ofstream shortiter;
    std::stringstream shortitrname;  // declared once, appended per jack as in the reference (:327,367-368)
    bool converged = false;
    for (unsigned mm = 0; mm < jacks; mm++) {
        if (muca_init_chains(ctx, rand_config ? MUCA_INIT_WEIGHT : MUCA_INIT_ORDERED, mm) != MUCA_OK)
            cli::die("init chains", ctx);
        std::vector<int32_t> ej(NUM_WORKERS * NofGPU), ed(NUM_WORKERS * NofGPU);
        if (muca_get_chain_state(ctx, ej.data(), ed.data(), nullptr, ej.size()) != MUCA_OK) cli::die("state", ctx);
        for (unsigned i = 0; i < NofGPU; i++) {  // :363-365
            std::cout << "E_DELTA : " << ed[(size_t)i * NUM_WORKERS] << std::endl;
            std::cout << "---------------------------------------- " << std::endl;
        }
        if (extrapolation)
            shortitrname << "./fss/L" << Ls << "/shortiter_gpu" << NofGPU << "_T050c" << NUM_WORKERS << "_M"
                         << initNUPDATES << "_therm" << therm_coeff << "N_Jack" << mm << "_extrapolated"
                         << extrapolation << ".txt";
        else
            shortitrname << "./fss/L" << Ls << "/shortiter_gpu" << NofGPU << "_T050c" << NUM_WORKERS << "_M"
                         << initNUPDATES << "_therm" << therm_coeff << "N_Jack" << mm << "_iterupdate1.01_rand.txt";
        shortiter.open(shortitrname.str().c_str());
        shortiter << "#iter width D_KL mcs_time memcpy_time accumulated_time NUPDATES acc_NUP" << std::endl;

        muca_run_opts ro{};
        ro.jack = mm;
        ro.starting_M = initNUPDATES;
        ro.therm = therm_coeff * N;
        ro.rule = recursion ? MUCA_UPDATE_RECURSION : MUCA_UPDATE_TRIVIAL;
        ro.hold_until_full = 0;
        ro.flat_minmean = opt.str("flat", "kl") == "minmean";
        ro.max_iter = (uint32_t)opt.num("max-iter", 0);
        ro.init_scheme = MUCA_INIT_WEIGHT;
        ro.reinit_chains = 0;
        ro.width_start = width;
        JackLog jl;
        jl.out = &shortiter;
        jl.N = N;
        muca_run_result res{};
        const muca_status st = muca_weight_run_stream(ctx, &ro, &res, on_iter, &jl);
        if (st != MUCA_OK && st != MUCA_ERR_NOT_CONVERGED) cli::die("weight run", ctx);
        shortiter.close();
        width = jl.width;
        converged = res.converged != 0;
        total_kernel[mm] = jl.total_kernel_ms;
        total_mem[mm] = res.total_mem_s * 1e3;
        total_run[mm] = res.total_run;
        Nwidth_time[mm] = jl.nwidth_time_s;
        Nwidth_step[mm] = jl.nwidth_step;
        if (converged) {  // :480-494
            total_kernel[mm] = total_kernel[mm] * 1e-3;
            std::cout << "D_KL is below 1e-4 !! " << std::endl;
            std::cout << "Total run : " << total_run[mm] << "" << "\tN_width time : " << Nwidth_time[mm]
                      << "\tMCS time : " << total_kernel[mm] << "\tMEM time : " << total_mem[mm]
                      << "\tRatio of time : " << Nwidth_time[mm] / total_kernel[mm] << std::endl;
            if (muca_get_weights(ctx, log_weight.data(), N + 1) != MUCA_OK) cli::die("get weights", ctx);
            std::ofstream weightfile;
            std::stringstream weightname;
            if (extrapolation)
                weightname << "./fss/L" << Ls << "/weight_gpu" << NofGPU << "_T050c" << NUM_WORKERS << "_M"
                           << initNUPDATES << "_therm" << therm_coeff << "N_JACK" << mm
                           << "_DKL1e-4_fromextrapolatedinit" << extrapolation << ".txt";
            else
                weightname << "./fss/L" << Ls << "/weight_gpu" << NofGPU << "_T050c" << NUM_WORKERS << "_M"
                           << initNUPDATES << "_therm" << therm_coeff << "N_JACK" << mm
                           << "_DKL1e-4_iterupdate1.01_rand.txt";
            weightfile.open(weightname.str().c_str());
            for (unsigned i = 0; i <= N; i++) weightfile << i << " " << std::setprecision(10) << log_weight[i] << std::endl;
            weightfile.close();
        } else {
            std::cout << "Noooo...not converged";
        }
        // --hist-dump: the jack's final weights beside its last iteration's
        // histogram, in the format of the reference's commented-out output
        // (:528-541), converged or not
        if (opt.has("hist-dump")) {
            std::vector<double> lnw((size_t)N + 1);
            std::vector<uint64_t> hist((size_t)N + 1);
            if (muca_get_weights(ctx, lnw.data(), N + 1) != MUCA_OK) cli::die("get weights", ctx);
            if (muca_get_histogram(ctx, hist.data(), N + 1) != MUCA_OK) cli::die("get histogram", ctx);
            std::string why;
            if (!cli::write_hist_dump("./fss/L" + Ls + "/E_Delta_multi_T050_JACK" + std::to_string(mm) + ".txt", lnw,
                                      hist, why))
                cli::die_io(why);
        }
    }

    // --save-chains: the chains' final lattices, for a production run to start from
    if (opt.has("save-chains")) {
        std::vector<int8_t> lat((size_t)NUM_WORKERS * NofGPU * N);
        if (muca_get_lattice(ctx, lat.data(), lat.size()) != MUCA_OK) cli::die("get lattice", ctx);
        std::string why;
        if (!cli::write_chains(opt.str("save-chains", ""), L, NUM_WORKERS * NofGPU, lat, why)) cli::die_chains(why);
    }

    // jackknife of the timings and step counts (:498-507), on the device
    double total_time_mean = 0, total_time_std = 0, total_memtime_mean = 0, total_memtime_std = 0;
    double Nwidth_time_mean = 0, Nwidth_time_std = 0, total_run_mean = 0, total_run_std = 0;
    double Nwidth_step_mean = 0, Nwidth_step_std = 0;
    for (unsigned i = 0; i < jacks; i++) {
        total_run_d[i] = (double)total_run[i];
        Nwidth_step_d[i] = (double)Nwidth_step[i];
    }
    muca_jackknife(ctx, total_kernel.data(), jacks, &total_time_mean, &total_time_std);
    muca_jackknife(ctx, total_mem.data(), jacks, &total_memtime_mean, &total_memtime_std);
    muca_jackknife(ctx, Nwidth_time.data(), jacks, &Nwidth_time_mean, &Nwidth_time_std);
    muca_jackknife(ctx, total_run_d.data(), jacks, &total_run_mean, &total_run_std);
    muca_jackknife(ctx, Nwidth_step_d.data(), jacks, &Nwidth_step_mean, &Nwidth_step_std);
    if (converged) {  // :509-524
        std::ofstream producefile;
        std::stringstream pdname;
        if (extrapolation)
            pdname << "./fss/L" << Ls << "/converge_result_gpu" << NofGPU << "_T050c" << NUM_WORKERS << "M"
                   << initNUPDATES << "_therm" << therm_coeff << "N_extrapolatedinit" << extrapolation << ".txt";
        else
            pdname << "./fss/L" << Ls << "/converge_result_gpu" << NofGPU << "_T050c" << NUM_WORKERS << "M"
                   << initNUPDATES << "_therm" << therm_coeff << "N_iterupdate1.01_rand.txt";
        producefile.open(pdname.str().c_str());
        producefile << "#total_time_mean" << " " << "total_time_std" << " " << "total_memtime_mean" << " "
                    << "total_memtime_std" << " " << "Nwidth_time_mean" << " " << "Nwidth_time_std" << " "
                    << "total_run_mean" << " " << "total_run_std" << " " << "Nwidth_step_mean" << " "
                    << "Nwidth_step_std" << std::endl;
        producefile << total_time_mean << " " << total_time_std << " " << " " << total_memtime_mean << " "
                    << total_memtime_std << " " << Nwidth_time_mean << " " << Nwidth_time_std << " "
                    << total_run_mean << " " << total_run_std << " " << Nwidth_step_mean << " " << Nwidth_step_std
                    << std::endl;
        producefile << "#total_mcstime" << " " << "total_memtime" << " " << "Nwidth_time" << " " << "total_run"
                    << " " << "Nwidth_step" << std::endl;
        for (unsigned i = 0; i < jacks; i++)
            producefile << total_kernel[i] << " " << total_mem[i] << " " << Nwidth_time[i] << " " << total_run[i]
                        << " " << Nwidth_step[i] << std::endl;
        producefile.close();
    }
    muca_destroy(ctx);
    return 0;
}
