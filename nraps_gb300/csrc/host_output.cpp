/*
 * host_output.cpp — the solver's output files and the input-file dispatch
 * (host only).
 *
 *   - nraps_format_f32/f64 give the text Rust's `Display` (`to_string()`)
 *     writes for a float, which is what plot_solution puts in every CSV field
 *     (src/plot_solution.rs:14-34): the shortest decimal digits that read back
 *     to the same value, placed positionally with no exponent ("1" for 1.0,
 *     "0.0000001", "100000000000000000000"), a leading '-' for negative values
 *     including -0.0, and "NaN", "inf", "-inf".  The digits come from
 *     std::to_chars in shortest scientific form (round-trip shortest, nearest
 *     to the exact value), then are laid out the positional way.
 *   - nraps_write_solution writes vars.csv, interface.csv and k_eff.csv like
 *     plot_solution (src/plot_solution.rs:36-58): one field per record in
 *     vars.csv (assembly length, cell count, generations); G flux rows, G
 *     assembly-average rows and the fission-source row in interface.csv;
 *     the k row and the k_fund row in k_eff.csv; ',' between fields and '\n'
 *     after each record (the csv crate's writer defaults).  The plot.py
 *     subprocess the reference starts afterwards (src/plot_solution.rs:60) is
 *     not started.
 *   - nraps_run_input is the dispatch of src/main.rs:332-364 with types
 *     that work: process_input, mesh_gen, then Monte Carlo with k = 1.0 when
 *     the file says `Solution = 1`, and the three output files.  The other
 *     solution kinds go to the deterministic solvers, which this library does
 *     not carry: NRAPS_ERR_UNSUPPORTED.
 */
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <system_error>
#include <vector>

#include "../../include/nraps_gpu.h"
#include "host_common.hpp"

namespace {

/* Lays out the shortest scientific form "d[.ddd]e[+-]x" positionally. */
template <class F>
std::string rust_display(F v) {
    if (std::isnan(v)) return "NaN";
    if (std::isinf(v)) return v < 0 ? "-inf" : "inf";
    std::string out;
    if (std::signbit(v)) {
        out.push_back('-');
        v = -v;
    }
    if (v == 0) {
        out.push_back('0');
        return out;
    }
    char buf[64];
    auto r = std::to_chars(buf, buf + sizeof(buf), v, std::chars_format::scientific);
    std::string sci(buf, r.ptr);
    size_t e = sci.find('e');
    std::string mant = sci.substr(0, e);
    int exp10 = std::atoi(sci.c_str() + e + 1);
    std::string digits;
    for (char c : mant)
        if (c != '.') digits.push_back(c);
    while (digits.size() > 1 && digits.back() == '0') digits.pop_back();
    /* value = 0.d1d2d3... x 10^(exp10 + 1) */
    int point = exp10 + 1;
    int nd = (int)digits.size();
    if (point <= 0) {
        out += "0.";
        out.append((size_t)(-point), '0');
        out += digits;
    } else if (point < nd) {
        out += digits.substr(0, (size_t)point);
        out.push_back('.');
        out += digits.substr((size_t)point);
    } else {
        out += digits;
        out.append((size_t)(point - nd), '0');
    }
    return out;
}

int put(const std::string& s, char* buf, uint64_t cap) {
    if (!buf || cap < s.size() + 1) return -1;
    std::memcpy(buf, s.data(), s.size());
    buf[s.size()] = '\0';
    return (int)s.size();
}

std::string join_path(const char* dir, const char* name) {
    std::string d = (dir && *dir) ? dir : ".";
    if (d.back() != '/') d.push_back('/');
    return d + name;
}

struct File {
    FILE* f = nullptr;
    explicit File(const std::string& p) : f(std::fopen(p.c_str(), "wb")) {}
    ~File() { if (f) std::fclose(f); }
};

void write_row(std::string& out, const float* v, uint64_t n) {
    for (uint64_t i = 0; i < n && v; ++i) {
        if (i) out.push_back(',');
        out += rust_display(v[i]);
    }
    out.push_back('\n');
}

int write_file(const std::string& path, const std::string& text) {
    File f(path);
    if (!f.f) {
        nraps_host::set_error("cannot open " + path + " for writing");
        return NRAPS_ERR_IO;
    }
    if (std::fwrite(text.data(), 1, text.size(), f.f) != text.size()) {
        nraps_host::set_error("short write to " + path);
        return NRAPS_ERR_IO;
    }
    return NRAPS_OK;
}

}  // namespace

extern "C" {

int nraps_format_f32(float v, char* buf, uint64_t cap) { return put(rust_display(v), buf, cap); }

int nraps_format_f64(double v, char* buf, uint64_t cap) { return put(rust_display(v), buf, cap); }

}  /* extern "C" */

namespace {

/* plot_solution's three files; the row lengths are the results' own
   (the deterministic solver has one k and no k_fund or fission source) */
int write_files(const char* dir, uint32_t G, uint64_t cells, uint64_t generations, double length,
                const float* flux, const float* avg, const float* fis, uint64_t n_fis, const float* k,
                uint64_t n_k, const float* k_fund, uint64_t n_kf) {
    std::string vars;
    vars += rust_display(length) + "\n";
    vars += std::to_string(cells) + "\n";
    vars += std::to_string(generations) + "\n";
    std::string iface;
    iface.reserve((size_t)(2 * G + 1) * cells * 12);
    for (uint32_t g = 0; g < G; ++g) write_row(iface, flux + (uint64_t)g * cells, cells);
    for (uint32_t g = 0; g < G; ++g) write_row(iface, avg + (uint64_t)g * cells, cells);
    write_row(iface, fis, n_fis);
    std::string keff;
    write_row(keff, k, n_k);
    write_row(keff, k_fund, n_kf);
    int s;
    if ((s = write_file(join_path(dir, "vars.csv"), vars)) != NRAPS_OK) return s;
    if ((s = write_file(join_path(dir, "interface.csv"), iface)) != NRAPS_OK) return s;
    return write_file(join_path(dir, "k_eff.csv"), keff);
}

}  // namespace

extern "C" {

int nraps_write_solution(const char* dir, const nraps_result* r, uint32_t energygroups, uint64_t cells,
                         uint64_t generations, double assembly_length) {
    /* plot_solution indexes results.flux[0] and results.assembly_average[0]
       (src/plot_solution.rs:17,24): it needs at least one group and all
       five arrays. */
    if (!r || !r->flux || !r->assembly_average || !r->fission_source || !r->k || !r->k_fund ||
        energygroups == 0) {
        nraps_host::set_error("nraps_write_solution: missing results or zero energy groups");
        return NRAPS_ERR_INVALID;
    }
    return write_files(dir, energygroups, cells, generations, assembly_length, r->flux, r->assembly_average,
                       r->fission_source, cells, r->k, generations, r->k_fund, generations);
}

int nraps_run_input(nraps_ctx* ctx, const char* input_path, const char* out_dir, nraps_stats* stats_out) {
    /* front-end failures are recorded per thread; move them onto the context */
    auto host_fail = [ctx](int code) {
        if (ctx) nraps_host::set_ctx_error(ctx, nraps_host::last_error());
        return code;
    };
    auto fail = [ctx](int code, const char* msg) {
        nraps_host::set_ctx_error(ctx, msg);
        return code;
    };
    nraps_input* in = nullptr;
    int s = nraps_process_input(input_path ? input_path : "./TestCaseC.txt", &in);
    if (s != NRAPS_OK) return host_fail(s);
    const bool monte_carlo = in->solution == 0;
    if (!monte_carlo && in->solver != 0) {
        nraps_input_free(in);
        return fail(NRAPS_ERR_UNSUPPORTED,
                    "Solution != 1 with the Gaussian, Jacobian or SR solver: the reference implements "
                    "only LinAlg (nalgebra_method) and returns empty results for the others");
    }
    if (monte_carlo && !ctx) {
        nraps_input_free(in);
        return fail(NRAPS_ERR_INVALID, "nraps_run_input: Solution = 1 runs Monte Carlo and needs a context");
    }
    nraps_meshbuf* mesh = nullptr;
    s = nraps_mesh_gen(in->matid, in->n_matid, &in->variables, &in->delta_x, &mesh);
    if (s != NRAPS_OK) {
        nraps_input_free(in);
        return host_fail(s);
    }
    nraps_problem p;
    s = nraps_problem_view(in, mesh, &p);
    if (s != NRAPS_OK) host_fail(s);
    if (s == NRAPS_OK && !monte_carlo) {
        /* (_, Solver::LinAlg) => nalgebra_method (src/main.rs:340-348) */
        const uint64_t G = in->variables.energygroups, nc = mesh->n_cells;
        std::vector<float> flux(G * nc), avg(G * nc);
        nraps_diffusion_info info{};
        s = nraps_diffusion_solve(&p, 0, flux.data(), avg.data(), &info);
        if (s != NRAPS_OK) {
            host_fail(s);
        } else {
            const float k1 = (float)info.k;
            if (stats_out) {
                std::memset(stats_out, 0, sizeof *stats_out);
                stats_out->k_mean = (double)k1;   /* the solver's one k; no histories */
            }
            const double length = (double)mesh->mesh_right[nc - 1];
            s = write_files(out_dir, (uint32_t)G, nc, in->variables.generations, length, flux.data(), avg.data(),
                            nullptr, 0, &k1, 1, nullptr, 0);
            if (s != NRAPS_OK) host_fail(s);
        }
        nraps_meshbuf_free(mesh);
        nraps_input_free(in);
        return s;
    }
    const uint64_t G = in->variables.energygroups, nc = mesh->n_cells, gens = in->variables.generations;
    std::vector<float> flux(G * nc), avg(G * nc), fis(nc), k(gens), kf(gens);
    nraps_stats st{};
    nraps_result r{};
    r.flux = flux.data();
    r.assembly_average = avg.data();
    r.fission_source = fis.data();
    r.k = k.data();
    r.k_fund = kf.data();
    r.stats = &st;
    if (s == NRAPS_OK) {
        p.k_new = 1.0f;
        s = nraps_solve(ctx, &p, &r);
    }
    if (s == NRAPS_OK) {
        /* plot_solution's assembly_length is an f64 (src/plot_solution.rs:12);
           the last cell's right edge is an f32 (src/main.rs:71), widened. */
        double length = nc ? (double)mesh->mesh_right[nc - 1] : 0.0;
        s = nraps_write_solution(out_dir, &r, (uint32_t)G, nc, gens, length);
        if (s != NRAPS_OK) host_fail(s);
    }
    if (s == NRAPS_OK && stats_out) *stats_out = st;
    nraps_meshbuf_free(mesh);
    nraps_input_free(in);
    return s;
}

} /* extern "C" */
