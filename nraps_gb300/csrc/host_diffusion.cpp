/*
 * host_diffusion.cpp — NRAPS's deterministic multigroup diffusion solver
 * (nalgebra_method, src/discrete.rs:169-356) on the host: an independent
 * sanity value for the Monte Carlo k, and what input files with
 * `Solution != 1` and the LinAlg solver run.
 *
 * Same model, same iteration, same bookkeeping as the reference, quirks
 * included; the arithmetic is FP64 and each group's system is solved as a
 * tridiagonal system instead of through an f32 dense inverse, so results
 * agree with the reference to its f32 rounding, not bit for bit.
 *
 *   matrix_gen (src/discrete.rs:4-97): per group a tridiagonal A with
 *     D(x) = inv_sigtr / (3 dx), face couplings 2 D_a D_b / (D_a + D_b),
 *     diagonal dx (sigt - sigma_s,g->g) plus the couplings; boundary rows
 *     2 D (1 - beta) with beta = 1 (reflective), 0.25 (vacuum) or the
 *     albedo formula.  Kept as the reference builds it: beta_r uses D of
 *     cell 1 (the function-scope `d_next`), and the last diagonal adds the
 *     coupling of faces 0|1 (the function-scope `d_nextcurr`).
 *   The reference stores A^-1 column-major and reads it back in chunks of n
 *     (src/discrete.rs:196-198), so row i of its `a_inv_matrix` is column i
 *     of A^-1 and the update is flux = A^-T (q/k + S); solved here as
 *     A^T y = q/k + S.
 *   q_gen (:99-123): q_g = chi_g dx sum_g' nu sigf_g' phi_g'.
 *   scat_calc (:125-147): out-scatter into g from the other groups with the
 *     current flux (groups updated in place, in order).
 *   Power iteration (:202-281): while delta_flux >= 1e-5 and
 *     delta_k >= 1e-6; delta_flux takes the max at the first and last cell
 *     but is overwritten by each interior cell, relative to the cell-0 flux
 *     of the group; k *= sum(q_new) / sum(q_old).
 *   Power normalisation (:283-329): flux * nu sigf flattened group-major
 *     and summed in chunks of G consecutive values, chunk c paired with
 *     cell c's width; flux *= 3565e6 / (1.6022e-13 * 200 * sum).
 *   average_assembly (:149-166): per-assembly mean written to each of its
 *     cells (cells / numass per assembly).
 * Cross-section indices are computed full width; the reference's u8
 * arithmetic (`matid + mattypes * g` as u8) would wrap when
 * MatTypes * EnergyGroups > 255.
 */
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/nraps_gpu.h"
#include "host_common.hpp"

namespace {

struct Tri {
    std::vector<double> lo, di, up;   /* A[i][i-1], A[i][i], A[i][i+1] */
};

/* Solves A^T y = b for tridiagonal A (Thomas algorithm on the transpose:
   its sub-diagonal is A's super-diagonal and vice versa). */
void solve_transposed(const Tri& A, const std::vector<double>& b, std::vector<double>& y,
                      std::vector<double>& c, std::vector<double>& d) {
    const size_t n = b.size();
    /* A^T[i][i-1] = A[i-1][i] = up[i-1], A^T[i][i+1] = A[i+1][i] = lo[i+1] */
    c.assign(n, 0.0);
    d.assign(n, 0.0);
    double den = A.di[0];
    c[0] = n > 1 ? A.lo[1] / den : 0.0;
    d[0] = b[0] / den;
    for (size_t i = 1; i < n; ++i) {
        const double sub = A.up[i - 1];
        den = A.di[i] - sub * c[i - 1];
        c[i] = (i + 1 < n) ? A.lo[i + 1] / den : 0.0;
        d[i] = (b[i] - sub * d[i - 1]) / den;
    }
    y.assign(n, 0.0);
    y[n - 1] = d[n - 1];
    for (size_t i = n - 1; i-- > 0;) y[i] = d[i] - c[i] * y[i + 1];
}

double beta_of(double bound, double d_a, double d_b) {
    if (bound == 1.0) return 1.0;
    if (bound == 0.0) return 0.25;
    const double r = (1.0 - bound) / (1.0 + bound);
    return (1.0 - 0.25 * (r * (1.0 / d_a))) / (1.0 + 0.25 * (r * (1.0 / d_b)));
}

}  // namespace

extern "C" {

int nraps_diffusion_solve(const nraps_problem* p, uint64_t max_iterations, float* flux_out,
                          float* assembly_average_out, nraps_diffusion_info* info) {
    if (!p || !p->mesh.matid || !p->mesh.delta_x || !p->xsdata.sigt || !p->xsdata.inv_sigtr ||
        !p->xsdata.scat_matrix || !p->xsdata.nut || !p->xsdata.sigf || !p->xsdata.chit) {
        nraps_host::set_error("nraps_diffusion_solve: missing problem arrays");
        return NRAPS_ERR_INVALID;
    }
    const uint64_t n = p->mesh.n_cells, G = p->variables.energygroups, M = p->variables.mattypes;
    if (n < 2 || G == 0 || M == 0) {
        nraps_host::set_error("nraps_diffusion_solve: needs at least two cells, one group and one material");
        return NRAPS_ERR_INVALID;
    }
    if (p->xsdata.n_xs < M * G || p->xsdata.n_scat < M * G * G) {
        nraps_host::set_error("nraps_diffusion_solve: cross-section arrays shorter than MatTypes x EnergyGroups");
        return NRAPS_ERR_INVALID;
    }
    const uint8_t* mat = p->mesh.matid;
    for (uint64_t i = 0; i < n; ++i)
        if (mat[i] >= M) {
            nraps_host::set_error("nraps_diffusion_solve: MatID beyond MatTypes");
            return NRAPS_ERR_INVALID;
        }
    const float* dxf = p->mesh.delta_x;
    const nraps_xsdata& x = p->xsdata;
    auto ix = [&](uint64_t m, uint64_t g) { return m + M * g; };
    auto s_gg = [&](uint64_t m, uint64_t g) { return (double)x.scat_matrix[G * G * m + G * g + g]; };
    auto D = [&](uint64_t i, uint64_t g) { return (1.0 / 3.0) * (double)x.inv_sigtr[ix(mat[i], g)] / (double)dxf[i]; };
    auto harm = [](double a, double b) { return (2.0 * a * b) / (a + b); };

    /* matrix_gen */
    std::vector<Tri> A(G);
    for (uint64_t g = 0; g < G; ++g) {
        Tri& t = A[g];
        t.lo.assign(n, 0.0); t.di.assign(n, 0.0); t.up.assign(n, 0.0);
        const double d_curr0 = D(0, g), d_next0 = D(1, g);
        const double dnc0 = harm(d_curr0, d_next0);
        const double bl = beta_of((double)p->variables.boundl, d_next0, d_curr0);
        t.di[0] = 2.0 * d_curr0 * (1.0 - bl) + (double)dxf[0] * ((double)x.sigt[ix(mat[0], g)] - s_gg(mat[0], g)) + dnc0;
        t.up[0] = -dnc0;
        for (uint64_t i = 1; i + 1 < n; ++i) {
            const double dc = D(i, g), dpc = harm(dc, D(i - 1, g)), dnc = harm(dc, D(i + 1, g));
            t.lo[i] = -dpc;
            t.di[i] = dpc + (double)dxf[i] * ((double)x.sigt[ix(mat[i], g)] - s_gg(mat[i], g)) + dnc;
            t.up[i] = -dnc;
        }
        const uint64_t l = n - 1;
        const double d_curr = D(l, g), dpc = harm(d_curr, D(l - 1, g));
        const double br = beta_of((double)p->variables.boundr, d_next0, d_curr);
        t.lo[l] = -dpc;
        t.di[l] = 2.0 * d_curr * (1.0 - br) + (double)dxf[l] * ((double)x.sigt[ix(mat[l], g)] - s_gg(mat[l], g)) + dnc0;
    }

    auto q_gen = [&](const std::vector<double>& phi, std::vector<double>& q) {
        q.assign(G * n, 0.0);
        for (uint64_t g = 0; g < G; ++g)
            for (uint64_t i = 0; i < n; ++i) {
                double s = 0.0;
                for (uint64_t e = 0; e < G; ++e)
                    s += (double)x.nut[ix(mat[i], e)] * (double)x.sigf[ix(mat[i], e)] * phi[e * n + i];
                q[g * n + i] = s * (double)dxf[i] * (double)x.chit[ix(mat[i], g)];
            }
    };
    auto total = [](const std::vector<double>& v) { double s = 0.0; for (double e : v) s += e; return s; };

    std::vector<double> phi(G * n, 1.0), q, q_old, b(n), y, cw, dw;
    q_gen(phi, q);
    double k = 1.0, delta_flux = 1.0, delta_k = 1.0;
    uint64_t it = 0;
    const uint64_t cap = max_iterations ? max_iterations : 100000;
    while (delta_flux >= 1e-5 && delta_k >= 1e-6 && it < cap) {
        q_old = q;
        for (uint64_t g = 0; g < G; ++g) {
            for (uint64_t i = 0; i < n; ++i) {
                double sc = 0.0;
                for (uint64_t e = 0; e < G; ++e)
                    if (e != g) sc += (double)x.scat_matrix[G * G * mat[i] + G * e + g] * phi[e * n + i] * (double)dxf[i];
                b[i] = q[g * n + i] * (1.0 / k) + sc;
            }
            solve_transposed(A[g], b, y, cw, dw);
            double* f = &phi[g * n];
            delta_flux = std::max(std::fabs((f[0] - y[0]) / f[0]), delta_flux);
            f[0] = y[0];
            for (uint64_t i = 1; i + 1 < n; ++i) {
                delta_flux = std::fabs((f[i] - y[i]) / f[0]);
                f[i] = y[i];
            }
            delta_flux = std::max(std::fabs((f[n - 1] - y[n - 1]) / f[0]), delta_flux);
            f[n - 1] = y[n - 1];
        }
        q_gen(phi, q);
        const double k_old = k;
        k = k_old * (total(q) / total(q_old));
        delta_k = std::fabs((k - k_old) / k_old);
        ++it;
    }
    const bool converged = !(delta_flux >= 1e-5 && delta_k >= 1e-6);

    /* power normalisation, chunked exactly as the reference chunks it */
    std::vector<double> flat(G * n);
    for (uint64_t e = 0; e < G; ++e)
        for (uint64_t i = 0; i < n; ++i)
            flat[e * n + i] = phi[e * n + i] * (double)x.nut[ix(mat[i], e)] * (double)x.sigf[ix(mat[i], e)];
    double psum = 0.0;
    for (uint64_t c = 0; c < n; ++c) {
        double ch = 0.0;
        for (uint64_t t = 0; t < G; ++t) ch += flat[c * G + t];
        psum += ch * (double)dxf[c];
    }
    const double power_constant = 3565e6 / (1.6022e-13 * 200.0 * psum);
    for (double& v : phi) v *= power_constant;

    if (flux_out)
        for (uint64_t i = 0; i < G * n; ++i) flux_out[i] = (float)phi[i];
    if (assembly_average_out) {
        std::memset(assembly_average_out, 0, G * n * sizeof(float));
        const uint64_t na = p->variables.numass ? p->variables.numass : 1, ma = n / na;
        for (uint64_t e = 0; e < G; ++e)
            for (uint64_t a = 0; a < na && ma > 0; ++a) {
                double s = 0.0;
                for (uint64_t i = a * ma; i < (a + 1) * ma; ++i) s += phi[e * n + i];
                const float avg = (float)(s / (double)ma);
                for (uint64_t i = a * ma; i < (a + 1) * ma; ++i) assembly_average_out[e * n + i] = avg;
            }
    }
    if (info) {
        info->k = k;
        info->iterations = it;
        info->converged = converged ? 1 : 0;
        info->delta_flux = delta_flux;
        info->delta_k = delta_k;
    }
    if (!converged) {
        nraps_host::set_error("nraps_diffusion_solve: iteration cap reached before convergence");
        return NRAPS_ERR_CAPPED;
    }
    return NRAPS_OK;
}

int nraps_diffusion_source(const nraps_problem* p, uint64_t n_sites, nraps_site* out, nraps_diffusion_info* info) {
    if (!p || !out || n_sites == 0 || !p->mesh.mesh_left) {
        nraps_host::set_error("nraps_diffusion_source: missing problem, output or sites");
        return NRAPS_ERR_INVALID;
    }
    const uint64_t n = p->mesh.n_cells, G = p->variables.energygroups, M = p->variables.mattypes;
    std::vector<float> flux(G * (n ? n : 1));
    nraps_diffusion_info di{};
    int s = nraps_diffusion_solve(p, 0, flux.data(), nullptr, &di);
    if (s != NRAPS_OK) return s;
    if (info) *info = di;
    const nraps_xsdata& x = p->xsdata;
    const uint8_t* mat = p->mesh.matid;
    /* fission density per cell and its running sum */
    std::vector<double> cdf(n + 1, 0.0);
    for (uint64_t c = 0; c < n; ++c) {
        double f = 0.0;
        for (uint64_t g = 0; g < G; ++g)
            f += (double)x.nut[mat[c] + M * g] * (double)x.sigf[mat[c] + M * g] * (double)flux[g * n + c];
        cdf[c + 1] = cdf[c] + std::max(0.0, f) * (double)p->mesh.delta_x[c];
    }
    const double total = cdf[n];
    if (!(total > 0.0)) {
        nraps_host::set_error("nraps_diffusion_source: the diffusion solution has no fission source");
        return NRAPS_ERR_INVALID;
    }
    /* chi CDFs as the transport kernels build them (f32 running sums) */
    std::vector<float> chi(M * G);
    for (uint64_t m = 0; m < M; ++m) {
        float run = 0.0f;
        for (uint64_t g = 0; g < G; ++g) { run += x.chit[m + M * g]; chi[m * G + g] = run; }
    }
    const double phi_golden = 0.6180339887498949;
    uint64_t c = 0;
    for (uint64_t i = 0; i < n_sites; ++i) {
        const double t = ((double)i + 0.5) / (double)n_sites * total;
        while (c + 1 < n && cdf[c + 1] <= t) ++c;
        const double w = cdf[c + 1] - cdf[c];
        double frac = w > 0.0 ? (t - cdf[c]) / w : 0.5;
        frac = std::min(std::max(frac, 0.0), 1.0);
        const float xs = (float)((double)p->mesh.mesh_left[c] + frac * (double)p->mesh.delta_x[c]);
        /* group: a low-discrepancy uniform through the cell material's chi */
        const double u = std::fmod(0.5 + (double)i * phi_golden, 1.0);
        const float* cd = &chi[(uint64_t)mat[c] * G];
        uint32_t g = 0;
        for (uint64_t e = 0; e < G; ++e) g += (cd[e] < (float)u) ? 1u : 0u;
        if (g > G - 1) g = (uint32_t)(G - 1);
        out[i].x = xs;
        out[i].cell = (uint32_t)c;
        out[i].group = g;
        out[i].pad = 0;
    }
    return NRAPS_OK;
}

} /* extern "C" */
