// yk_run.cpp -- the run protocol of code/src/main.cu:73-516 on top of the C
// ABI: burn-in (:302-316), epsBar measurement and rescale (:325-352), the
// export loop (:368-484) with its stdout lines and the files slice.dat,
// data.csv and traces.csv, and the SIGUSR2 early finish (:66-75, :425-428).
// Checkpoints (field, Philox step, Langevin time, epsBar) are written at the
// end of a run and read back when io.resume = true (the reference parses
// io.startFileName / io.resume but never uses them, main.cu:146-157).
#include <atomic>
#include <chrono>
#include <cmath>
#include <csignal>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <string>
#include <vector>

#include "yk_host.h"

namespace {

std::atomic<bool> g_early_finish(false);

void on_sigusr2(int) { g_early_finish = true; }

struct CkptHeader {
    char magic[8];
    int32_t Nt, Nx;
    int64_t step;
    double time, eps_bar;
};

}  // namespace

extern "C" {

int yk_checkpoint_save(yk_ctx* ctx, int chain, const char* path, double eps_bar)
{
    const int V = yk_ctx_volume(ctx, chain);
    if (V <= 0) return YK_EINVAL;
    std::vector<double> phi(V);
    if (int rc = yk_get_field_host(ctx, chain, phi.data())) return rc;
    yk_obs obs;
    if (int rc = yk_observables(ctx, chain, &obs)) return rc;
    int64_t step = 0;
    if (int rc = yk_get_step(ctx, chain, &step)) return rc;
    int Nt = 0, Nx = 0;
    yk_ctx_shape(ctx, chain, &Nt, &Nx);
    CkptHeader h;
    std::memcpy(h.magic, "YKCKPT1", 8);
    h.Nt = Nt;
    h.Nx = Nx;
    h.step = step;
    h.time = obs.t;
    h.eps_bar = eps_bar;
    // a chain with pions appends pi_1..3 (3V doubles) and marks the header
    std::vector<double> pi(3 * (size_t)V);
    double* dpi = nullptr;
    const bool pions = yk_pions_device(ctx, chain, &dpi) == YK_OK;
    if (pions) {
        if (int rc = yk_get_pions_host(ctx, chain, pi.data())) return rc;
        h.magic[6] = 'P';
    }
    FILE* f = std::fopen(path, "wb");
    if (!f) {
        yk::set_error("cannot write checkpoint %s", path);
        return YK_EIO;
    }
    bool ok = std::fwrite(&h, sizeof(h), 1, f) == 1 && std::fwrite(phi.data(), sizeof(double), V, f) == (size_t)V;
    if (ok && pions) ok = std::fwrite(pi.data(), sizeof(double), pi.size(), f) == pi.size();
    std::fclose(f);
    if (!ok) {
        yk::set_error("short write to %s", path);
        return YK_EIO;
    }
    return YK_OK;
}

int yk_checkpoint_load(yk_ctx* ctx, int chain, const char* path, double* eps_bar)
{
    const int V = yk_ctx_volume(ctx, chain);
    if (V <= 0) return YK_EINVAL;
    FILE* f = std::fopen(path, "rb");
    if (!f) {
        yk::set_error("cannot read checkpoint %s", path);
        return YK_EIO;
    }
    CkptHeader h;
    std::vector<double> phi(V), pi(3 * (size_t)V);
    double* dpi = nullptr;
    const bool pions = yk_pions_device(ctx, chain, &dpi) == YK_OK;
    bool ok = std::fread(&h, sizeof(h), 1, f) == 1 &&
              std::memcmp(h.magic, pions ? "YKCKPTP" : "YKCKPT1", 8) == 0 && (int64_t)h.Nt * h.Nx == V &&
              std::fread(phi.data(), sizeof(double), V, f) == (size_t)V;
    if (ok && pions) ok = std::fread(pi.data(), sizeof(double), pi.size(), f) == pi.size();
    std::fclose(f);
    if (!ok) {
        yk::set_error("checkpoint %s does not match the lattice (or its pions)", path);
        return YK_EIO;
    }
    if (int rc = yk_set_field_host(ctx, chain, phi.data())) return rc;
    if (pions)
        if (int rc = yk_set_pions_host(ctx, chain, pi.data())) return rc;
    if (int rc = yk_set_step(ctx, chain, h.step)) return rc;
    if (int rc = yk_set_time(ctx, chain, h.time)) return rc;
    if (eps_bar) *eps_bar = h.eps_bar;
    return YK_OK;
}

int yk_run_toml(const char* toml_path, const char* out_dir)
{
    yk_params p;
    if (int rc = yk_params_from_toml(toml_path, &p)) return rc;
    std::map<std::string, std::string> kv;
    std::string perr;
    yk::parse_toml(toml_path, kv, perr);
    auto sget = [&](const char* k, const char* d) {
        auto it = kv.find(k);
        return it == kv.end() ? std::string(d) : it->second;
    };
    const std::string dir = (out_dir && *out_dir) ? std::string(out_dir) + "/" : std::string();
    const std::string slice_name = sget("io.timeSliceFileName", "slice.dat");
    const std::string config_name = sget("io.configFileName", "test.hdf");
    const std::string start_name = sget("io.startFileName", "");
    const bool resume = sget("io.resume", "false") == "true";

    std::signal(SIGUSR2, on_sigusr2);
    std::printf("Nt: %d Nx: %d\n", p.Nt, p.Nx);
    {
        std::ifstream in(toml_path);
        std::string line;
        while (std::getline(in, line)) std::printf("#%s\n", line.c_str());
        std::printf("\n\n");
    }
    yk_action act;
    yk_derive_action(&p, &act);
    yk_ctx* ctx = nullptr;
    if (int rc = yk_ctx_create(&p, 1, &ctx)) return rc;
    const int V = p.Nt * p.Nx;
    double eps_bar = p.average_epsilon;
    if (resume && !start_name.empty()) {
        if (int rc = yk_checkpoint_load(ctx, 0, (dir + start_name).c_str(), &eps_bar)) {
            yk_ctx_destroy(ctx);
            return rc;
        }
        yk_set_eps_bar(ctx, 0, eps_bar);
    }
    std::FILE* datafile = std::fopen((dir + "data.csv").c_str(), "w");
    std::FILE* tracefile = std::fopen((dir + "traces.csv").c_str(), "w");
    if (!datafile || !tracefile) {
        yk::set_error("cannot open output files in %s", dir.c_str());
        yk_ctx_destroy(ctx);
        return YK_EIO;
    }
    std::fprintf(datafile, "corr\n");
    std::fprintf(tracefile, "tr,sigma,phi\n");
    std::printf("\n");
    std::fflush(stdout);

    int rc = YK_OK;
    yk_obs obs;
    // one export block: steps until the accumulated eps reaches ExportTime
    // [gpu] learned_layers > 0: after thermalisation a network of that many
    // layers is trained on pairs from the chain's own CG, and the steps that
    // follow solve with it (flexible preconditioned CG in FP64 refinement)
    bool learned = false;
    auto export_block = [&](double& t_out, double& eps_last) -> int {
        double t = 0.0;
        while (t < p.export_time) {
            if (learned) {
                yk_solve_stats st;
                if (int r = yk_langevin_step_learned(ctx, 1, 1, &st)) return r;
            } else if (int r = yk_langevin_step(ctx, 1)) {
                return r;
            }
            if (int r = yk_observables(ctx, 0, &obs)) return r;
            if (obs.status == YK_ENAN || obs.status == YK_ETIMEOUT) {
                yk::set_error("step failed with status %d", obs.status);
                return obs.status;
            }
            t += obs.eps;
            eps_last = obs.eps;
        }
        t_out = t;
        return YK_OK;
    };

    double t_blk = 0.0, eps_last = p.average_epsilon;
    for (int burn = 0; burn < p.burn_count && rc == YK_OK; ++burn) rc = export_block(t_blk, eps_last);
    if (rc == YK_OK) std::printf("Thermalization done!\n");
    if (rc == YK_OK && p.learned_layers > 0 && p.yukawa_coupling == 0.0)
        std::printf("Learned preconditioner: not used (gpu.learned_layers = %d, but yukawa_coupling = 0: "
                    "no fermion solves)\n", p.learned_layers);
    if (rc == YK_OK && p.learned_layers > 0 && p.yukawa_coupling != 0.0) {
        rc = yk_net_setup(ctx, 0, p.learned_layers, 7, -1.0);
        yk_net_train_cfg cfg = {4, 5, 4, 400, 4, 2e-3, 3};
        yk_net_train_stats ts;
        if (rc == YK_OK) rc = yk_net_train(ctx, 0, &cfg, &ts);
        if (rc == YK_OK) {
            std::printf("Learned preconditioner: %d layers, %d pairs, loss %.4f -> %.4f (%.0f ms)\n",
                        p.learned_layers, ts.pairs, ts.loss0, ts.loss1, ts.ms);
            learned = true;
        }
    }
    double elapsed = 0.0;
    if (rc == YK_OK && p.measure_drift_count > 0) {
        double eps_sum = 0.0;
        int nmeas = 0;
        while (elapsed < p.measure_drift_count * p.export_time && rc == YK_OK) {
            rc = export_block(t_blk, eps_last);
            elapsed += t_blk;
            eps_sum += eps_last;
            nmeas++;
        }
        if (nmeas > 0) {
            eps_sum /= nmeas;
            std::printf("#Average eps during drift measurement = %g\n", eps_sum);
            eps_bar *= eps_bar / eps_sum;   // main.cu:349
        }
    }
    if (rc == YK_OK) {
        yk_set_eps_bar(ctx, 0, eps_bar);
        std::printf("Drift measuring done!\n");
    }
    std::FILE* slicefile = std::fopen((dir + slice_name).c_str(), "w");
    elapsed = 0.0;
    int nmeas = 0;
    double avg_mag = 0.0, trace = 0.0;
    std::vector<double> slices(p.Nt), corr(p.Nt);
    const auto t0 = std::chrono::high_resolution_clock::now();
    while (rc == YK_OK && elapsed < p.max_langevin_time) {
        rc = export_block(t_blk, eps_last);
        if (rc) break;
        elapsed += t_blk;
        double avg = obs.sum_phi;   // gpuMagnetisation
        if ((rc = yk_time_slices(ctx, 0, slices.data()))) break;
        if (slicefile) {
            for (int tt = 0; tt < p.Nt; ++tt) std::fprintf(slicefile, "%g\t", slices[tt] / p.Nx);
            std::fprintf(slicefile, "\n\n");
        }
        std::printf("%g\t%g\t", elapsed, eps_last);
        if (!p.use_mass) avg /= act.sq2kappa;
        std::printf("%g\t", avg / V);
        const double sum2 = avg * avg;
        if (g_early_finish) {
            std::printf("#Early termination signal received.\n#Wrapping up.\n");
            elapsed = p.max_langevin_time + 1.0;
        }
        nmeas++;
        avg_mag += std::fabs(avg);
        std::printf("abs. mag: %g \t cond: %g \t partial avg: %g\n", std::fabs(avg) / V, std::fabs(trace) / V,
                    avg_mag / nmeas / V);
        if (p.pions) {
            // pion extension: |<pi>| = |sum_n pi(n)| / V (not in the reference's output)
            const double pm = std::sqrt(obs.sum_pi[0] * obs.sum_pi[0] + obs.sum_pi[1] * obs.sum_pi[1] +
                                        obs.sum_pi[2] * obs.sum_pi[2]);
            std::printf("#pions: |<pi>|: %g \t <|pi|^2>: %g\n", pm / V, obs.sum_pi2 / V);
        }
        // fermion correlator from a point source (main.cu:441-469)
        yk_solve_stats st;
        int r2 = yk_correlator(ctx, 0, corr.data(), &st);
        if (r2 && r2 != YK_ENOCONV) { rc = r2; break; }
        for (int nt = 0; nt < p.Nt; ++nt) std::fprintf(datafile, "%g\n", corr[nt]);
        // condensate from a fresh force (main.cu:471-483)
        double cond = 0.0;
        r2 = yk_condensate(ctx, 0, &cond, &st);
        if (r2 && r2 != YK_ENOCONV) { rc = r2; break; }
        trace = cond * V;
        std::fprintf(tracefile, "%g,%g,%g\n", trace / V, avg / V, std::sqrt(sum2) / V);
        std::fflush(stdout);
    }
    const auto t1 = std::chrono::high_resolution_clock::now();
    if (rc == YK_OK) {
        std::printf("Final abs. magnetisation: %g\n", nmeas ? avg_mag / nmeas / V : 0.0);
        std::printf("#Number of measurements: %d\n", nmeas);
        std::printf("#Run time for main loop: %g s\n", std::chrono::duration<double>(t1 - t0).count());
        rc = yk_checkpoint_save(ctx, 0, (dir + config_name + ".ckpt").c_str(), eps_bar);
    }
    if (slicefile) std::fclose(slicefile);
    std::fclose(datafile);
    std::fclose(tracefile);
    yk_ctx_destroy(ctx);
    std::fflush(stdout);
    return rc;
}

}  // extern "C"
