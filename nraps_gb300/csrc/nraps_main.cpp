/*
 * nraps_main.cpp — the command-line program over libnraps_gb300.so: the
 * reference's main (src/main.rs:332-369) with the Monte Carlo dispatch
 * restored.  It reads an input file (default ./TestCaseC.txt, the file the
 * reference opens at src/process_input.rs:86), runs the Monte Carlo solver
 * when the file says Solution = 1 and the deterministic diffusion solver
 * (LinAlg) otherwise, writes vars.csv, interface.csv and k_eff.csv, and
 * prints the run time in milliseconds.
 *
 *   nraps [input] [-o out_dir] [--mode compat|physics|bank]
 *         [--form plain|event] [--fp32] [--seed N] [--device N]
 *
 * The defaults reproduce the reference's algorithm (COMPAT, FP64 plain
 * history kernel); `--mode bank --form event` runs the fission-bank power
 * iteration on the event-based Woodcock engine.
 */
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "../../include/nraps_gpu.h"

static int usage(const char* argv0) {
    std::fprintf(stderr,
                 "usage: %s [input] [-o out_dir] [--mode compat|physics|bank] [--form plain|event]\n"
                 "          [--fp32] [--seed N] [--device N]\n",
                 argv0);
    return 2;
}

int main(int argc, char** argv) {
    std::string input = "./TestCaseC.txt", out_dir = ".";
    nraps_opts o;
    nraps_opts_default(&o);
    bool have_input = false;
    for (int i = 1; i < argc; ++i) {
        std::string a = argv[i];
        auto next = [&](void) -> const char* { return i + 1 < argc ? argv[++i] : nullptr; };
        if (a == "-o") {
            const char* v = next();
            if (!v) return usage(argv[0]);
            out_dir = v;
        } else if (a == "--mode") {
            const char* v = next();
            if (!v) return usage(argv[0]);
            std::string m = v;
            if (m == "compat") o.mode = NRAPS_MODE_COMPAT;
            else if (m == "physics") o.mode = NRAPS_MODE_PHYSICS;
            else if (m == "bank") o.mode = NRAPS_MODE_BANK;
            else return usage(argv[0]);
        } else if (a == "--form") {
            const char* v = next();
            if (!v) return usage(argv[0]);
            std::string f = v;
            if (f == "plain") o.tracking = NRAPS_TRACK_SURFACE;
            else if (f == "event") { o.tracking = NRAPS_TRACK_WOODCOCK; o.precision = NRAPS_PREC_FP32; }
            else return usage(argv[0]);
        } else if (a == "--fp32") {
            o.precision = NRAPS_PREC_FP32;
        } else if (a == "--seed") {
            const char* v = next();
            if (!v) return usage(argv[0]);
            o.seed = std::strtoull(v, nullptr, 10);
        } else if (a == "--device") {
            const char* v = next();
            if (!v) return usage(argv[0]);
            o.device = std::atoi(v);
        } else if (a == "-h" || a == "--help") {
            return usage(argv[0]);
        } else if (!have_input && !a.empty() && a[0] != '-') {
            input = a;
            have_input = true;
        } else {
            return usage(argv[0]);
        }
    }
    auto t0 = std::chrono::steady_clock::now();
    /* a GPU context only for Monte Carlo inputs (Solution = 1) */
    nraps_input* probe = nullptr;
    int s = nraps_process_input(input.c_str(), &probe);
    if (s != NRAPS_OK) {
        const char* m = nraps_last_error(nullptr);
        std::fprintf(stderr, "nraps: %s\n", (m && *m) ? m : nraps_status_string(s));
        return 1;
    }
    const bool monte_carlo = probe->solution == 0;
    nraps_input_free(probe);
    nraps_ctx* ctx = nullptr;
    if (monte_carlo) {
        s = nraps_create(&ctx, &o);
        if (s != NRAPS_OK) {
            const char* m = nraps_last_error(nullptr);
            std::fprintf(stderr, "nraps: %s\n", (m && *m) ? m : nraps_status_string(s));
            return 1;
        }
    }
    nraps_stats st;
    std::memset(&st, 0, sizeof st);
    s = nraps_run_input(ctx, input.c_str(), out_dir.c_str(), &st);
    if (s != NRAPS_OK) {
        const char* m = nraps_last_error(ctx);
        std::fprintf(stderr, "nraps: %s\n", (m && *m) ? m : nraps_status_string(s));
        if (ctx) nraps_destroy(ctx);
        return 1;
    }
    if (ctx) nraps_destroy(ctx);
    auto ms = std::chrono::duration_cast<std::chrono::milliseconds>(std::chrono::steady_clock::now() - t0).count();
    std::printf("Run was completed in %lld milliseconds \n", (long long)ms);
    if (st.histories) std::printf("k = %.6f +- %.6f over the active generations\n", st.k_mean, st.k_sigma);
    else std::printf("%.10f\n", st.k_mean);   /* nalgebra_method prints its k ({:.10}) */
    return 0;
}
