/*
 * tables.cpp — packs one slab problem into the device table layout.
 *
 * Compiled with -ffp-contract=off: the derived tables (inv_sigtr recomputed
 * in FP64, nu*sigf, cumulative chi, transport-corrected scatter CDFs) must
 * round exactly like the CPU restatement that checks the kernels.
 * inv_sigtr follows src/process_input.rs:152-156 (1/(sigt - mu*sigs)); the
 * cumulative chi follows energy() (src/mc_code.rs:19-30).
 */
#include "tables.hpp"
#include "nr_math.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>

namespace {
size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }
}

template <class T>
int build_tables(const nraps_problem& p, std::vector<unsigned char>& blob, TableLayout& L,
                 std::string& err) {
    const nraps_variables& v = p.variables;
    const uint64_t M = v.mattypes, G = v.energygroups, nc = p.mesh.n_cells, nx = M * G;
    if (M == 0 || G == 0 || nc == 0) { err = "empty problem (mattypes, energygroups or cells is 0)"; return 1; }
    if (G > 16) { err = "at most 16 energy groups are supported"; return 1; }
    if (p.xsdata.n_xs < nx || p.xsdata.n_scat < nx * G) { err = "cross-section arrays shorter than MatTypes*EnergyGroups"; return 1; }
    if (p.n_fuel == 0 || !p.fuel_indices) { err = "no fuel cells (fuel_indices is empty)"; return 1; }
    for (uint64_t c = 0; c < nc; ++c)
        if (p.mesh.matid[c] >= M) { err = "mesh matid out of range of MatTypes"; return 1; }
    for (uint64_t i = 0; i < p.n_fuel; ++i)
        if (p.fuel_indices[i] >= nc) { err = "fuel index out of range of the mesh"; return 1; }

    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off = align_up(off + bytes); return o; };
    L.sigt = take(nx * sizeof(T)); L.sigs = take(nx * sizeof(T)); L.siga = take(nx * sizeof(T));
    L.inv_sigtr = take(nx * sizeof(T)); L.nsf = take(nx * sizeof(T)); L.nsf_sigtr = take(nx * sizeof(T));
    L.pabs = take(nx * sizeof(T)); L.scat = take(nx * G * sizeof(T)); L.chi_cdf = take(nx * sizeof(T));
    L.phys_cdf = take(nx * G * sizeof(T));
    L.left = take(nc * sizeof(T)); L.right = take(nc * sizeof(T)); L.dx = take(nc * sizeof(T));
    L.mat = take(nc); L.fuel = take(p.n_fuel * 8);
    L.nsf64 = take(nx * 8); L.dx64 = take(nc * 8);
    L.total = off;
    blob.assign(off, 0);
    auto arr = [&](size_t o) { return reinterpret_cast<T*>(blob.data() + o); };

    T* sigt = arr(L.sigt); T* sigs = arr(L.sigs); T* siga = arr(L.siga);
    T* inv = arr(L.inv_sigtr); T* nsf = arr(L.nsf); T* nsfs = arr(L.nsf_sigtr); T* pabs = arr(L.pabs);
    T* scat = arr(L.scat); T* chi = arr(L.chi_cdf); T* phys = arr(L.phys_cdf);
    double* nsf64 = reinterpret_cast<double*>(blob.data() + L.nsf64);
    for (uint64_t i = 0; i < nx; ++i) {
        sigt[i] = (T)p.xsdata.sigt[i]; sigs[i] = (T)p.xsdata.sigs[i]; siga[i] = (T)p.xsdata.siga[i];
        if (sizeof(T) == 4) inv[i] = (T)p.xsdata.inv_sigtr[i];
        else inv[i] = T(1) / ((T)p.xsdata.sigt[i] - (T)p.xsdata.mu[i] * (T)p.xsdata.sigs[i]);
        nsf[i] = (T)p.xsdata.nut[i] * (T)p.xsdata.sigf[i];
        nsfs[i] = nsf[i] * inv[i];
        pabs[i] = siga[i] * inv[i];
        nsf64[i] = (double)p.xsdata.nut[i] * (double)p.xsdata.sigf[i];
    }
    for (uint64_t i = 0; i < nx * G; ++i) scat[i] = (T)p.xsdata.scat_matrix[i];
    for (uint64_t m = 0; m < M; ++m) {
        T c = 0;
        for (uint64_t g = 0; g < G; ++g) { c += (T)p.xsdata.chit[m + M * g]; chi[m * G + g] = c; }
    }
    for (uint64_t m = 0; m < M; ++m)
        for (uint64_t g = 0; g < G; ++g) {
            uint64_t xs = m + M * g;
            T cum[16]; T c = 0;
            for (uint64_t e = 0; e < G; ++e) {
                T s = scat[G * G * m + G * g + e];
                if (e == g) s = s - (T)p.xsdata.mu[xs] * sigs[xs];
                if (s < T(0)) s = T(0);
                c = c + s; cum[e] = c;
            }
            for (uint64_t e = 0; e < G; ++e) phys[(m * G + g) * G + e] = (c > T(0)) ? cum[e] / c : T(1);
        }
    T* left = arr(L.left); T* right = arr(L.right); T* dx = arr(L.dx);
    double* dx64 = reinterpret_cast<double*>(blob.data() + L.dx64);
    for (uint64_t c = 0; c < nc; ++c) {
        left[c] = (T)p.mesh.mesh_left[c]; right[c] = (T)p.mesh.mesh_right[c];
        dx[c] = (T)p.mesh.delta_x[c]; dx64[c] = (double)p.mesh.delta_x[c];
    }
    std::memcpy(blob.data() + L.mat, p.mesh.matid, nc);
    std::memcpy(blob.data() + L.fuel, p.fuel_indices, p.n_fuel * 8);
    uint64_t inu = std::min<uint64_t>(M, nx - 1);     /* nut of material 0, group 1 */
    L.conv_const = 3565e6 * 36.2 /
        (200e6 * 1.602176634e-19 * (double)p.xsdata.nut[inu] * (double)p.mesh.mesh_right[nc - 1]);
    return 0;
}

template int build_tables<float>(const nraps_problem&, std::vector<unsigned char>&, TableLayout&, std::string&);
template int build_tables<double>(const nraps_problem&, std::vector<unsigned char>&, TableLayout&, std::string&);

int build_event_tables(const nraps_problem& p, EvHostTables& t, std::string& err) {
    const nraps_variables& v = p.variables;
    const uint64_t M = v.mattypes, G = v.energygroups, nc = p.mesh.n_cells;
    if (M == 0 || G == 0 || nc == 0) { err = "empty problem (mattypes, energygroups or cells is 0)"; return 1; }
    if (G > 16) { err = "at most 16 energy groups are supported"; return 1; }
    if (M > 255) { err = "at most 255 materials are supported"; return 1; }
    if (nc >= (1ULL << 27)) { err = "at most 2^27 cells are supported"; return 1; }
    if (p.xsdata.n_xs < M * G || p.xsdata.n_scat < M * G * G) { err = "cross-section arrays shorter than MatTypes*EnergyGroups"; return 1; }
    if (p.n_fuel == 0 || !p.fuel_indices) { err = "no fuel cells (fuel_indices is empty)"; return 1; }
    t.M = (uint32_t)M; t.G = (uint32_t)G; t.nc = (uint32_t)nc; t.nfuel = (uint32_t)p.n_fuel;
    t.boundl = v.boundl; t.boundr = v.boundr;
    const nraps_xsdata& x = p.xsdata;
    t.xs.assign(M * G * 4, 0.f);
    std::vector<float> sigtr(M * G);
    for (uint64_t m = 0; m < M; ++m)
        for (uint64_t g = 0; g < G; ++g) {
            uint64_t i = m + M * g;
            float st = (float)((double)x.sigt[i] - (double)x.mu[i] * (double)x.sigs[i]);
            sigtr[m * G + g] = st;
            float* X = &t.xs[(m * G + g) * 4];
            X[0] = st;
            X[1] = st > 0.f ? x.siga[i] / st : 1.f;
            X[2] = st > 0.f ? (x.nut[i] * x.sigf[i]) / st : 0.f;
            X[3] = st > 0.f ? 1.0f / st : 0.f;
        }
    t.scdf.assign(M * G * G, 1.f);
    for (uint64_t m = 0; m < M; ++m)
        for (uint64_t g = 0; g < G; ++g) {
            uint64_t i = m + M * g;
            float cum[16]; float c = 0.f;
            for (uint64_t e = 0; e < G; ++e) {
                float s = x.scat_matrix[G * G * m + G * g + e];
                if (e == g) s = s - x.mu[i] * x.sigs[i];
                if (s < 0.f) s = 0.f;
                c = c + s; cum[e] = c;
            }
            for (uint64_t e = 0; e < G; ++e) t.scdf[(m * G + g) * G + e] = (c > 0.f) ? cum[e] / c : 1.f;
        }
    /* one uniform decides absorption and the scatter group together */
    t.ocdf.assign(M * G * G, 1.f);
    for (uint64_t j = 0; j < M * G; ++j) {
        const float pa = t.xs[j * 4 + 1];
        const float q = 1.0f - pa;
        t.ocdf[j * G] = pa;
        for (uint64_t e = 1; e < G; ++e) t.ocdf[j * G + e] = pa + q * t.scdf[j * G + e - 1];
    }
    t.chicdf.assign(M * G, 0.f);
    for (uint64_t m = 0; m < M; ++m) {
        float c = 0.f;
        for (uint64_t g = 0; g < G; ++g) { c += x.chit[m + M * g]; t.chicdf[m * G + g] = c; }
    }
    /* regions */
    t.rleft.clear(); t.rmat.clear(); t.rfirst.clear(); t.rncell.clear(); t.rinvdx.clear();
    std::vector<bool> present(M, false);
    for (uint64_t c = 0; c < nc; ++c) {
        uint8_t m = p.mesh.matid[c];
        if (m >= M) { err = "mesh matid out of range of MatTypes"; return 1; }
        present[m] = true;
        bool start = c == 0 || m != p.mesh.matid[c - 1] ||
                     std::memcmp(&p.mesh.delta_x[c], &p.mesh.delta_x[c - 1], 4) != 0;
        if (start) {
            t.rleft.push_back(p.mesh.mesh_left[c]);
            t.rmat.push_back(m);
            t.rfirst.push_back((uint32_t)c);
            t.rncell.push_back(1);
            t.rinvdx.push_back((float)(1.0 / (double)p.mesh.delta_x[c]));
        } else {
            t.rncell.back()++;
        }
    }
    t.R = (uint32_t)t.rmat.size();
    if (t.R > 65535) { err = "at most 65535 material regions are supported"; return 1; }
    t.rleft.push_back(p.mesh.mesh_right[nc - 1]);
    t.L = t.rleft[t.R];
    if (!(t.L > 0.f) || t.rleft[0] != 0.f) { err = "mesh must start at 0 and have positive length"; return 1; }
    t.maj.assign(2 * G, 0.f);
    for (uint64_t g = 0; g < G; ++g) {
        float mj = 0.f;
        for (uint64_t m = 0; m < M; ++m)
            if (present[m]) {
                if (!(sigtr[m * G + g] > 0.f)) { err = "sigt - mu*sigs must be positive for every material in the mesh"; return 1; }
                mj = std::max(mj, sigtr[m * G + g]);
            }
        t.maj[g] = mj;
        t.maj[G + g] = 1.0f / mj;
    }
    double wmin = 1e300;
    for (uint32_t r = 0; r < t.R; ++r) {
        double w = (double)t.rleft[r + 1] - (double)t.rleft[r];
        if (!(w > 0.0)) { err = "material region of zero width"; return 1; }
        wmin = std::min(wmin, w);
    }
    /* bins no wider than half the narrowest region: at most one region
       boundary per bin, unless the 16384-bin cap binds */
    uint64_t want = (uint64_t)std::ceil(2.0 * (double)t.L / wmin);
    uint32_t nb = 16;
    while (nb < want && nb < 16384) nb <<= 1;
    t.nbins = nb;
    t.inv_binw = (float)((double)nb / (double)t.L);
    /* The device maps x to bin (int)(x * inv_binw) (one f32 multiply,
       truncation, clamp to [0, nb-1]); that map never decreases with x.  So
       every x >= boundary B lies in a bin >= bin(B), and every x in a bin
       > bin(B) is >= B: the first region a bin can hold is the number of
       boundaries whose own bin lies below it. */
    auto bin_of = [&](float xv) -> uint32_t {
        float f = xv * t.inv_binw;
        int b = (int)f;
        b = b < 0 ? 0 : (b >= (int)nb ? (int)nb - 1 : b);
        return (uint32_t)b;
    };
    std::vector<uint32_t> first_region(nb, 0), boundaries(nb, 0);
    for (uint32_t r = 1; r < t.R; ++r) boundaries[bin_of(t.rleft[r])]++;
    uint32_t below = 0;
    for (uint32_t b = 0; b < nb; ++b) { first_region[b] = below; below += boundaries[b]; }
    t.bins.assign(2 * (size_t)nb, 0);
    for (uint32_t b = 0; b < nb; ++b) {
        const uint32_t r0 = first_region[b];
        const float x1 = r0 + 1 < t.R ? t.rleft[r0 + 1] : std::numeric_limits<float>::infinity();
        uint32_t xb;
        std::memcpy(&xb, &x1, 4);
        t.bins[2 * b] = xb;
        t.bins[2 * b + 1] = r0 | (boundaries[b] > 1 ? 0x80000000u : 0u);
    }
    t.rdat.assign(4 * ((size_t)t.R + 1), 0.f);
    for (uint32_t r = 0; r <= t.R; ++r) {
        float* d = &t.rdat[4 * (size_t)r];
        d[0] = t.rleft[r];
        if (r < t.R) {
            d[1] = t.rinvdx[r];
            std::memcpy(&d[2], &t.rfirst[r], 4);
            std::memcpy(&d[3], &t.rncell[r], 4);
        }
    }
    t.fuel.resize(p.n_fuel);
    for (uint64_t i = 0; i < p.n_fuel; ++i) {
        if (p.fuel_indices[i] >= nc) { err = "fuel index out of range of the mesh"; return 1; }
        t.fuel[i] = (uint32_t)p.fuel_indices[i];
    }
    t.cleft.assign(p.mesh.mesh_left, p.mesh.mesh_left + nc);
    t.cdx.assign(p.mesh.delta_x, p.mesh.delta_x + nc);
    t.cmat.assign(p.mesh.matid, p.mesh.matid + nc);
    t.nsf64.resize(M * G);
    for (uint64_t i = 0; i < M * G; ++i) t.nsf64[i] = (double)x.nut[i] * (double)x.sigf[i];
    t.dx64.resize(nc);
    t.inv_dx64.resize(nc);
    for (uint64_t c = 0; c < nc; ++c) {
        t.dx64[c] = (double)p.mesh.delta_x[c];
        t.inv_dx64[c] = 1.0 / t.dx64[c];
    }
    t.inv_st64.resize(M * G);
    t.kq.resize(M * G);
    for (uint64_t j = 0; j < M * G; ++j) {
        t.inv_st64[j] = (double)t.xs[j * 4 + 3];
        t.kq[j] = nr_fix((double)t.xs[j * 4 + 2]);
    }
    uint64_t inu = std::min<uint64_t>(M, M * G - 1);
    t.conv_const = 3565e6 * 36.2 /
        (200e6 * 1.602176634e-19 * (double)x.nut[inu] * (double)p.mesh.mesh_right[nc - 1]);
    return 0;
}
