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

#include <algorithm>
#include <cstring>

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
