"""Seeded synthetic slab problems for the benchmark workloads.

Cross-section generator (per material and group, seeded):
  sigt ~ U[0.2, 2.0] 1/cm; scatter ratio c ~ U[0.5, 0.95]; sigs = c*sigt;
  siga = sigt - sigs; scattering row g -> g' nonzero only for g' >= g-1,
  downscatter-dominant, summing to sigs; mu-bar = 0 (isotropic);
  nu = 2.43; sigf nonzero in fuel only, sigf <= siga, scaled so that the
  deterministic k of the slab is 1.0; chi = [0.97, 0.03, 0, ...] in fuel.
Materials follow the reference's numbering: fuel = 0, water = 2 (material 1
is a copy of the fuel, unused), so MatTypes = 3.

"Deterministic k" is defined by `diffusion_k`: FP64 multigroup diffusion,
cell-centred finite differences on the tally mesh, Marshak vacuum boundaries
(or zero-current for reflective ones), the full multigroup loss operator
factorised once, and a power iteration on the fission source.  The 12,500 cm
scale_stress slab has a dominance ratio so close to one that a power
iteration crawls; `diffusion_k_large` finds the same eigenvalue with Arnoldi
iterations on a cell-major, banded factorisation.

Workloads (1D slab, vacuum boundaries unless stated):
  plain_small     4 groups, 10 fuel regions of 1.0 cm alternating with 11 water
                  regions of 1.5 cm, 20/30 cells per fuel/water region, built
                  through mesh_gen (MPWR/2 cells trimmed at each edge: 500 cells,
                  25.0 cm), 10k histories, 50 inactive + 100 active, FP64.
  single_large    the same slab and generator, 80/120 cells per region
                  (2,000 cells), 1M histories, 50 + 200 generations.
  batched         256 instances: regions U{4..64}, groups U{2..8}, widths
                  U[0.5, 3.0] cm, histories log-uniform [10k, 500k].
  scale_stress    8 groups, 10,000 regions with widths U[0.5, 2.0] cm,
                  200,000 tally cells, 10M histories, 20 + 50 generations.
"""
from __future__ import annotations

import math

import numpy as np

from .abi import ProblemArrays

NU = 2.43
FUEL, WATER = 0, 2


def xs_set(rng: np.random.Generator, G: int):
    """Cross sections of (fuel, water) for G groups: dict of (M*G) arrays."""
    M = 3
    sigt = np.zeros(M * G); sigs = np.zeros(M * G); siga = np.zeros(M * G)
    scat = np.zeros(M * G * G)
    frac_f = np.zeros(G)
    for m in (FUEL, WATER):
        for g in range(G):
            st = rng.uniform(0.2, 2.0)
            c = rng.uniform(0.5, 0.95)
            sigt[m + M * g] = st
            sigs[m + M * g] = c * st
            siga[m + M * g] = st - c * st
            w = np.zeros(G)
            if g >= 1:
                w[g - 1] = rng.uniform(0.0, 0.05)
            w[g] = rng.uniform(0.3, 0.6)
            for gp in range(g + 1, G):
                w[gp] = rng.uniform(0.2, 0.5) * 0.5 ** (gp - g - 1)
            if g == G - 1:
                w[g] += 0.4
            w /= w.sum()
            scat[G * G * m + G * g: G * G * m + G * g + G] = w * c * st
    for g in range(G):
        frac_f[g] = rng.uniform(0.3, 0.8)
    # material 1: copy of fuel (unused slot, keeps the reference numbering)
    for g in range(G):
        sigt[1 + M * g] = sigt[M * g]; sigs[1 + M * g] = sigs[M * g]; siga[1 + M * g] = siga[M * g]
    scat[G * G: 2 * G * G] = scat[0: G * G]
    chi = np.zeros(M * G)
    chi_f = np.zeros(G)
    chi_f[0] = 0.97 if G > 1 else 1.0
    if G > 1:
        chi_f[1] = 0.03
    for g in range(G):
        chi[M * g] = chi_f[g]
        chi[1 + M * g] = chi_f[g]
    sigf_shape = np.zeros(M * G)
    for g in range(G):
        sigf_shape[M * g] = frac_f[g] * siga[M * g]
        sigf_shape[1 + M * g] = sigf_shape[M * g]
    return dict(M=M, G=G, sigt=sigt, sigs=sigs, siga=siga, scat=scat, chi=chi, sigf_shape=sigf_shape)


def diffusion_k(mat, dx, xs, sigf, boundl=0.0, boundr=0.0, tol=1e-9, max_outer=5000):
    """FP64 multigroup diffusion k of a slab: cell-centred finite differences,
    Marshak vacuum (zero-current reflective) boundaries, the full multigroup
    loss operator factorised once (sparse LU), power iteration on the fission
    source."""
    from scipy.sparse import coo_matrix
    from scipy.sparse.linalg import splu
    M, G = xs["M"], xs["G"]
    mat = np.asarray(mat, np.int64)
    h = np.asarray(dx, np.float64)
    n = h.size
    sigt = xs["sigt"]; scat = xs["scat"]; chi = xs["chi"]
    rows, cols, vals = [], [], []
    nsf = np.zeros((G, n)); chic = np.zeros((G, n))
    for g in range(G):
        idx = mat + M * g
        D = 1.0 / (3.0 * sigt[idx])
        dc = 2.0 * D[:-1] * D[1:] / (h[:-1] * D[1:] + h[1:] * D[:-1])
        diag = (sigt[idx] - scat[G * G * mat + G * g + g]) * h
        diag[:-1] += dc
        diag[1:] += dc
        diag[0] += 0.0 if boundl > 0 else 2.0 * D[0] / (4.0 * D[0] + h[0])
        diag[-1] += 0.0 if boundr > 0 else 2.0 * D[-1] / (4.0 * D[-1] + h[-1])
        base = g * n
        i = np.arange(n)
        rows += [base + i, base + i[:-1], base + i[1:]]
        cols += [base + i, base + i[1:], base + i[:-1]]
        vals += [diag, -dc, -dc]
        for gp in range(G):                       # in-scatter gp -> g
            if gp != g:
                rows.append(base + i); cols.append(gp * n + i)
                vals.append(-scat[G * G * mat + G * gp + g] * h)
        nsf[g] = NU * sigf[idx]
        chic[g] = chi[idx]
    A = coo_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                   shape=(G * n, G * n)).tocsc()
    lu = splu(A)
    phi = np.ones(G * n)
    k = 1.0
    fs = (nsf * phi.reshape(G, n)).sum(0) * h
    for _ in range(max_outer):
        src = (chic * fs).reshape(-1) / k
        phi = lu.solve(src)
        fs_new = (nsf * phi.reshape(G, n)).sum(0) * h
        k_new = k * fs_new.sum() / fs.sum()
        fs = fs_new
        if abs(k_new - k) < tol:
            k = k_new
            break
        k = k_new
    return float(k)


def diffusion_k_large(mat, dx, xs, sigf, boundl=0.0, boundr=0.0, tol=1e-9):
    """The same diffusion k as `diffusion_k` for slabs too long for a power
    iteration (the 12,500 cm scale-stress slab: its dominance ratio is so
    close to one that hundreds of outer iterations barely move k): unknowns
    ordered cell-major, so the loss operator is block tridiagonal with G x G
    blocks and its LU keeps to the band; the dominant eigenvalue of
    loss^-1 * fission found by implicitly restarted Arnoldi (ARPACK)."""
    from scipy.sparse import coo_matrix
    from scipy.sparse.linalg import LinearOperator, eigs, splu
    M, G = xs["M"], xs["G"]
    mat = np.asarray(mat, np.int64)
    h = np.asarray(dx, np.float64)
    n = h.size
    sigt = xs["sigt"]; scat = xs["scat"]; chi = xs["chi"]
    rows, cols, vals = [], [], []
    nsf = np.zeros((n, G)); chic = np.zeros((n, G))
    i = np.arange(n)
    for g in range(G):
        idx = mat + M * g
        D = 1.0 / (3.0 * sigt[idx])
        dc = 2.0 * D[:-1] * D[1:] / (h[:-1] * D[1:] + h[1:] * D[:-1])
        diag = (sigt[idx] - scat[G * G * mat + G * g + g]) * h
        diag[:-1] += dc
        diag[1:] += dc
        diag[0] += 0.0 if boundl > 0 else 2.0 * D[0] / (4.0 * D[0] + h[0])
        diag[-1] += 0.0 if boundr > 0 else 2.0 * D[-1] / (4.0 * D[-1] + h[-1])
        rows += [i * G + g, i[:-1] * G + g, i[1:] * G + g]
        cols += [i * G + g, i[1:] * G + g, i[:-1] * G + g]
        vals += [diag, -dc, -dc]
        for gp in range(G):                       # in-scatter gp -> g
            if gp != g:
                rows.append(i * G + g); cols.append(i * G + gp)
                vals.append(-scat[G * G * mat + G * gp + g] * h)
        nsf[:, g] = NU * sigf[idx]
        chic[:, g] = chi[idx]
    A = coo_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                   shape=(G * n, G * n)).tocsc()
    lu = splu(A, permc_spec="NATURAL")

    def apply(x):
        fs = (nsf * x.reshape(n, G)).sum(1) * h
        return lu.solve((chic * fs[:, None]).reshape(-1))

    op = LinearOperator((G * n, G * n), matvec=apply, dtype=np.float64)
    w = eigs(op, k=1, which="LM", tol=tol, v0=np.ones(G * n), ncv=40, return_eigenvectors=False)
    return float(w[0].real)


def _mesh_from_regions(region_mat, region_width, cells_per_region):
    mats, dxs, lefts, rights = [], [], [], []
    left = np.float32(0.0)
    for m, w, nc in zip(region_mat, region_width, cells_per_region):
        d = np.float32(np.float32(w) / np.float32(nc))
        for _ in range(int(nc)):
            mats.append(m); dxs.append(d); lefts.append(left)
            right = np.float32(left + d)
            rights.append(right)
            left = right
    mats = np.array(mats, np.uint8)
    fuel = np.nonzero((mats == 0) | (mats == 1))[0].astype(np.uint64)
    return mats, np.array(dxs, np.float32), np.array(lefts, np.float32), np.array(rights, np.float32), fuel


def infinite_k(mats, dxs, xs, sigf):
    """k-infinity of the volume-homogenised slab (FP64 G x G eigenproblem):
    the deterministic k of a slab so wide that leakage is negligible."""
    M, G = xs["M"], xs["G"]
    mats = np.asarray(mats, np.int64)
    w = np.asarray(dxs, np.float64)
    vol = np.array([w[mats == m].sum() for m in range(M)]) / w.sum()
    A = np.zeros((G, G)); F = np.zeros((G, G))
    for m in range(M):
        if vol[m] == 0:
            continue
        for g in range(G):
            A[g, g] += vol[m] * xs["sigt"][m + M * g]
            for gp in range(G):
                A[gp, g] -= vol[m] * xs["scat"][G * G * m + G * g + gp]
            for gp in range(G):
                F[gp, g] += vol[m] * xs["chi"][m + M * gp] * NU * sigf[m + M * g]
    ev = np.linalg.eigvals(np.linalg.solve(A, F))
    return float(np.max(ev.real))


def _scale_fission(xs, mats, dxs, boundl, boundr, method="diffusion"):
    """sigf = shape / k(shape), clamped at siga: the diffusion k of the slab is
    then 1 (recomputed when the clamp bites).  k is linear in a common scale
    of sigf, so one eigenvalue solve sets it."""
    shape = xs["sigf_shape"]
    if method == "infinite":
        k1 = infinite_k(mats, dxs, xs, shape)
        sigf = np.minimum(shape / k1, xs["siga"])
        return sigf, infinite_k(mats, dxs, xs, sigf)
    solve = diffusion_k_large if method == "diffusion_large" else diffusion_k
    k1 = solve(mats, dxs, xs, shape, boundl, boundr)
    sigf = shape / k1
    sigf = np.minimum(sigf, xs["siga"])
    k = solve(mats, dxs, xs, sigf, boundl, boundr) if np.any(sigf < shape / k1) else 1.0
    return sigf, k


def slab_reference_layout(seed: int, G: int = 4, mpfr: int = 20, mpwr: int = 30, histories: int = 10_000,
                          inactive: int = 50, active: int = 100, n_fuel_regions: int = 10,
                          fuel_width: float = 1.0, water_width: float = 1.5, name: str = "") -> ProblemArrays:
    """Alternating fuel/water slab in the reference input format's geometry.

    The mesh is what mesh_gen builds from MatID = 2 0 2 ... 0 2 with
    NumAss = 1: MPWR/2 cells are trimmed from each edge water region.
    """
    rng = np.random.default_rng(seed)
    xs = xs_set(rng, G)
    matid = [WATER]
    for _ in range(n_fuel_regions):
        matid += [FUEL, WATER]
    dxf = np.float32(np.float32(fuel_width) / np.float32(mpfr))
    dxw = np.float32(np.float32(water_width) / np.float32(mpwr))
    temp = []
    for m in matid:
        temp += [m] * (mpfr if m in (0, 1) else mpwr)
    half = mpwr // 2
    temp = temp[half: len(temp) - half]
    mats = np.array(temp, np.uint8)
    dxs = np.where((mats == 0) | (mats == 1), dxf, dxw).astype(np.float32)
    lefts = np.zeros(mats.size, np.float32); rights = np.zeros(mats.size, np.float32)
    left = np.float32(0.0)
    for i in range(mats.size):
        lefts[i] = left
        rights[i] = np.float32(left + dxs[i])
        left = rights[i]
    fuel = np.nonzero((mats == 0) | (mats == 1))[0].astype(np.uint64)
    sigf, kdet = _scale_fission(xs, mats, dxs, 0.0, 0.0)
    M = xs["M"]
    p = ProblemArrays(
        mattypes=M, energygroups=G, generations=inactive + active, histories=histories, skip=inactive,
        sigt=xs["sigt"], sigs=xs["sigs"], mu=np.zeros(M * G), siga=xs["siga"], sigf=sigf,
        nut=np.where(sigf > 0, NU, 0.0), chit=xs["chi"], scat=xs["scat"], matid=mats, delta_x=dxs,
        mesh_left=lefts, mesh_right=rights, fuel_indices=fuel, boundl=0.0, boundr=0.0, numass=1,
        numrods=n_fuel_regions, roddia=fuel_width, rodpitch=water_width, mpfr=mpfr, mpwr=mpwr,
        dx_fuel=float(dxf), dx_water=float(dxw), k_new=1.0, name=name)
    p.k_deterministic = kdet
    p.input_matid = np.array(matid, np.uint8)
    return p


def plain_small(seed: int = 1) -> ProblemArrays:
    return slab_reference_layout(seed, G=4, mpfr=20, mpwr=30, histories=10_000, inactive=50, active=100,
                                 name="plain_small: 4 groups, 500 cells, 10k histories, 50+100 generations")


def single_large(seed: int = 1) -> ProblemArrays:
    return slab_reference_layout(seed, G=4, mpfr=80, mpwr=120, histories=1_000_000, inactive=50, active=200,
                                 name="single_large: 4 groups, 2000 cells, 1M histories, 50+200 generations")


def random_slab(rng: np.random.Generator, n_regions: int, G: int, wmin: float, wmax: float,
                cells_per_region: int, histories: int, inactive: int, active: int,
                name: str = "", k_method: str = "diffusion") -> ProblemArrays:
    xs = xs_set(rng, G)
    region_mat = [WATER if i % 2 == 0 else FUEL for i in range(n_regions)]
    if FUEL not in region_mat:
        region_mat[-1] = FUEL
    widths = rng.uniform(wmin, wmax, n_regions)
    mats, dxs, lefts, rights, fuel = _mesh_from_regions(region_mat, widths, [cells_per_region] * n_regions)
    sigf, kdet = _scale_fission(xs, mats, dxs, 0.0, 0.0, k_method)
    M = xs["M"]
    p = ProblemArrays(
        mattypes=M, energygroups=G, generations=inactive + active, histories=histories, skip=inactive,
        sigt=xs["sigt"], sigs=xs["sigs"], mu=np.zeros(M * G), siga=xs["siga"], sigf=sigf,
        nut=np.where(sigf > 0, NU, 0.0), chit=xs["chi"], scat=xs["scat"], matid=mats, delta_x=dxs,
        mesh_left=lefts, mesh_right=rights, fuel_indices=fuel, boundl=0.0, boundr=0.0, numass=1,
        numrods=0, roddia=1.0, rodpitch=1.0, mpfr=cells_per_region, mpwr=cells_per_region,
        dx_fuel=float(dxs[fuel[0]]), dx_water=float(dxs[0]), k_new=1.0, name=name)
    p.k_deterministic = kdet
    return p


def batched(seed: int = 1, n: int = 256, cells_per_region: int = 10, inactive: int = 20,
            active: int = 20) -> list[ProblemArrays]:
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        R = int(rng.integers(4, 65))
        G = int(rng.integers(2, 9))
        N = int(round(math.exp(rng.uniform(math.log(1e4), math.log(5e5)))))
        out.append(random_slab(rng, R, G, 0.5, 3.0, cells_per_region, N, inactive, active,
                               name=f"batched[{i}]: {R} regions, {G} groups, {N} histories"))
    return out


_SCALE_STRESS = {}


def scale_stress(seed: int = 1, histories: int = 10_000_000) -> ProblemArrays:
    """nu*sigf scaled by the slab's diffusion k (Arnoldi on the 1.6M-unknown
    operator, ~15 s; cached per seed within a process)."""
    if seed not in _SCALE_STRESS:
        rng = np.random.default_rng(seed)
        _SCALE_STRESS[seed] = random_slab(
            rng, 10_000, 8, 0.5, 2.0, 20, 10_000_000, 20, 50, k_method="diffusion_large",
            name="scale_stress: 8 groups, 10000 regions, 200000 cells, 10M histories, 20+50")
    p = _SCALE_STRESS[seed]
    return p if histories == p.histories else p.with_(histories=histories)


def write_input_file(p: ProblemArrays, path: str, solution: int = 1) -> None:
    """Write a problem built by slab_reference_layout in the reference's
    input-file format (keys of src/process_input.rs)."""
    M, G = p.mattypes, p.energygroups

    def f(v):
        return repr(float(np.float32(v)))

    lines = ["# NRAPS input file (synthetic slab, written by nraps_gb300.synth)",
             f"Solution = {solution}", "Analk = 1", f"MatTypes = {M}", f"EnergyGroups = {G}",
             "solver = 0", f"Generations = {p.generations}", f"Histories = {p.histories}",
             f"Skip = {p.skip}", "NumAss = 1", f"NumRods = {p.numrods}",
             f"RodDia = {f(p.roddia)}", f"RodPitch = {f(p.roddia + p.rodpitch)}",
             f"MPFR = {p.mpfr}", f"MPWR = {p.mpwr}", f"BoundL = {f(p.boundl)}", f"BoundR = {f(p.boundr)}",
             "", "XSData"]
    for key, arr in (("SigT", p.sigt), ("SigS", p.sigs), ("mu", p.mu), ("SigA", p.siga), ("SigF", p.sigf),
                     ("nuT", p.nut), ("ChiT", p.chit)):
        for g in range(G):
            lines.append(f"    {key} = " + " ".join(f(arr[m + M * g]) for m in range(M)))
    for m in range(M):
        lines.append("    Scat = " + " ".join(f(v) for v in p.scat[G * G * m: G * G * (m + 1)]))
    lines.append("ConfigSets")
    lines.append("    MatID = " + " ".join(str(int(v)) for v in p.input_matid))
    lines.append("END")
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")
