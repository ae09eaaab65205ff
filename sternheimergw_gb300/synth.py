"""Deterministic synthetic Sternheimer systems (the five benchmark shapes).

Units: Rydberg atomic units throughout.  Kinetic energy is |k+G|^2 Ry with G in
bohr^-1 (Quantum ESPRESSO's g2kin convention); V_loc, D_ii, eigenvalues and
frequencies are in Ry (eV inputs are divided by ``RY_EV``).

A system holds everything the reference's callers set up before calling the
solver (solve_linter.f90:288-337 and green.f90:38-93 via QE init_us_2/g2_kin):
  * the k and k+q G-spheres (Miller indices, sphere -> box index ``nl``),
    ordered by |k+G|^2 with ties broken by Miller index, so the integer maps are
    bit-exact on every machine (exact integer keys);
  * the FFT box (nr1, nr2, nr3), V_loc(r) on it (real);
  * Kleinman-Bylander projectors beta(k+q+G) and D_ii;
  * occupied states at k (psi_v, eps_v) and at k+q (evq) from a dense FP64
    diagonalisation of the same H;
  * alpha_pv (the generator's rule: 2 (eps_max - eps_min) over the occupied
    bands, at least 1e-2 Ry, restating the role of QE setup_alpha_pv);
  * perturbations Delta V = exp(i (q+G_p).r) and frequency lists.
"""
from __future__ import annotations

import math
from fractions import Fraction

import numpy as np

RY_EV = 13.605693122994

# --- lattices (vectors in units of a; reciprocal vectors in units of 2 pi / a) ---
_FCC_A = np.array([[-0.5, 0.0, 0.5], [0.0, 0.5, 0.5], [-0.5, 0.5, 0.0]])
_FCC_B = np.array([[-1, -1, 1], [1, 1, 1], [-1, 1, -1]], dtype=np.int64)
_SC_A = np.eye(3)
_SC_B = np.eye(3, dtype=np.int64)
_DIAMOND8 = np.array([[0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0],
                      [.25, .25, .25], [.25, .75, .75], [.75, .25, .75], [.75, .75, .25]])


def good_fft_size(n_min: int) -> int:
    """Smallest 2,3,5-smooth integer >= n_min."""
    n = max(int(n_min), 1)
    while True:
        m = n
        for p in (2, 3, 5):
            while m % p == 0:
                m //= p
        if m == 1:
            return n
        n += 1


def fft_grid_for(alat: float, avec: np.ndarray, ecut_rho: float) -> tuple:
    """QE-style smooth grid: nr_i >= 2 * |a_i| sqrt(ecutrho)/(2 pi) + 1, 2,3,5-smooth."""
    gmax = math.sqrt(ecut_rho)
    out = []
    for i in range(3):
        ai = np.linalg.norm(avec[i]) * alat
        out.append(good_fft_size(int(2 * math.floor(gmax * ai / (2 * math.pi)) + 1)))
    return tuple(out)


def _rational_vec(v, denom=1000):
    return [Fraction(x).limit_denominator(denom) for x in v]


def sphere(bmat: np.ndarray, kvec_frac, alat: float, ecut: float, nr):
    """G-vectors with |k+G|^2 <= ecut (Ry, bohr^-2).

    kvec_frac: k in units of 2 pi / a as exact Fractions.  Returns Miller
    indices (npw, 3) int32 sorted by |k+G|^2 then Miller index, the box index
    nl, and |k+G|^2.  The cutoff test and the ordering use exact integer keys.
    """
    D = 1
    for f in kvec_frac:
        D = D * f.denominator // math.gcd(D, f.denominator)
    kD = np.array([int(f * D) for f in kvec_frac], dtype=np.int64)
    tpiba = 2 * math.pi / alat
    # |k+G|^2 (bohr^-2) = tpiba^2 * key / D^2 with key = |D k + D (m.B)|^2 (exact integer)
    thr = ecut * D * D / (tpiba * tpiba)
    bnorm = min(np.linalg.norm(bmat, axis=1))
    mmax = int(math.ceil((math.sqrt(ecut) / tpiba + np.abs(np.array([float(f) for f in kvec_frac])).sum()) * 2 / max(bnorm, 1e-9))) + 2
    r = np.arange(-mmax, mmax + 1, dtype=np.int64)
    m = np.stack(np.meshgrid(r, r, r, indexing="ij"), -1).reshape(-1, 3)
    gD = kD[None, :] + D * (m @ bmat)
    key = (gD * gD).sum(1)
    sel = key <= thr
    m, key = m[sel], key[sel]
    order = np.lexsort((m[:, 2], m[:, 1], m[:, 0], key))
    m, key = m[order], key[order]
    nl = (np.mod(m[:, 0], nr[0]) + nr[0] * (np.mod(m[:, 1], nr[1]) + nr[1] * np.mod(m[:, 2], nr[2]))).astype(np.int32)
    g2 = key.astype(np.float64) * (tpiba * tpiba) / (D * D)
    return m.astype(np.int32), nl, g2


def _cart(bmat, m, kvec, alat):
    return (2 * math.pi / alat) * (m.astype(np.float64) @ bmat.astype(np.float64) + kvec[None, :])


def gaussian_vloc(rng, nr, bmat, alat, rms=0.5):
    """Real Gaussian random field on the box, G-amplitude ~ exp(-|G|^2/8), zero mean, given rms (Ry)."""
    nr1, nr2, nr3 = nr
    w = rng.standard_normal((nr3, nr2, nr1))
    wg = np.fft.fftn(w)
    f = [np.fft.fftfreq(n, 1.0 / n) for n in (nr1, nr2, nr3)]
    m1, m2, m3 = np.meshgrid(f[0], f[1], f[2], indexing="ij")  # (nr1, nr2, nr3)
    mm = np.stack([m1, m2, m3], -1).reshape(-1, 3)
    g = (2 * math.pi / alat) * (mm @ bmat.astype(np.float64))
    filt = np.exp(-(g * g).sum(1) / 8.0).reshape(nr1, nr2, nr3).transpose(2, 1, 0)
    filt[0, 0, 0] = 0.0
    v = np.fft.ifftn(wg * filt).real
    v *= rms / math.sqrt(np.mean(v * v))
    return np.ascontiguousarray(v.reshape(-1))  # index i1 + nr1*(i2 + nr2*i3)


def kb_projectors(rng, kpg_cart, tau_cart, omega):
    """s + 3 p per atom: exp(-|k+G|^2/4) Y_lm (-i)^l exp(-i (k+G).tau) / sqrt(Omega)."""
    npw = kpg_cart.shape[0]
    q2 = (kpg_cart ** 2).sum(1)
    qn = np.sqrt(q2)
    radial = np.exp(-q2 / 4.0) / math.sqrt(omega)
    safe = np.where(qn > 0, qn, 1.0)
    ylm = [np.full(npw, 1.0 / math.sqrt(4 * math.pi))]
    c1 = math.sqrt(3.0 / (4 * math.pi))
    for ax in range(3):
        ylm.append(np.where(qn > 0, c1 * kpg_cart[:, ax] / safe, 0.0))
    cols = []
    for t in tau_cart:
        phase = np.exp(-1j * (kpg_cart @ t))
        for l, y in zip((0, 1, 1, 1), ylm):
            cols.append(radial * y * ((-1j) ** l) * phase)
    vkb = np.stack(cols, 1)
    dvan = rng.uniform(-2.0, 2.0, vkb.shape[1])
    return vkb, dvan


def box_to_g(vrs, nr):
    """V(G) on the whole box (fwfft normalisation), shape (nr3, nr2, nr1)."""
    nr1, nr2, nr3 = nr
    return np.fft.fftn(vrs.reshape(nr3, nr2, nr1)) / (nr1 * nr2 * nr3)


def dense_h(miller, g2kin, vrs, nr, vkb, dvan):
    """Dense H[G,G'] = g2kin delta + V(G-G' mod box) + sum_i beta_i(G) D_i beta_i(G')^*.

    The (G - G') mod box index makes this exactly the FFT-based operator.
    """
    nr1, nr2, nr3 = nr
    vg = box_to_g(vrs, nr)
    d = miller[:, None, :] - miller[None, :, :]
    h = vg[np.mod(d[..., 2], nr3), np.mod(d[..., 1], nr2), np.mod(d[..., 0], nr1)]
    h = h + np.diag(g2kin)
    h = h + (vkb * dvan[None, :]) @ vkb.conj().T
    return 0.5 * (h + h.conj().T)


def lowest_states(h, nocc):
    """Lowest eigenpairs; each vector's phase is fixed so that its largest
    component is real and positive (LAPACK builds differ in the phase they return)."""
    w, v = np.linalg.eigh(h)
    v = v[:, :nocc].copy()
    for j in range(nocc):
        k = int(np.argmax(np.abs(v[:, j])))
        v[:, j] *= np.conj(v[k, j]) / abs(v[k, j])
    return w[:nocc].copy(), np.asfortranarray(v)


def dense_states(mill, nl, g2kin, vrs, nr, vkb, dvan, nocc):
    """Lowest nocc eigenpairs of the dense FP64 H (numpy eigh)."""
    return lowest_states(dense_h(mill, g2kin, vrs, nr, vkb, dvan), nocc)


def make_system(alat, lattice, ecut, nocc, seed, nr=None, qvec=(0.1, 0.0, 0.0), n_pert=1,
                kvec=(0.0, 0.0, 0.0), eigensolver=None):
    """Build one synthetic system (see module docstring).

    eigensolver(mill, nl, g2kin, vrs, nr, vkb, dvan, nocc) -> (eps, psi) gives
    the occupied states (default: dense eigh); large systems pass an iterative
    solver (sternheimergw_gb300.eigen)."""
    rng = np.random.default_rng(seed)
    if lattice == "fcc":
        avec, bmat, tau = _FCC_A, _FCC_B, np.array([[0, 0, 0], [0.25, 0.25, 0.25]])
        omega = alat ** 3 / 4.0
    elif lattice == "sc8":
        avec, bmat, tau = _SC_A, _SC_B, _DIAMOND8
        omega = alat ** 3
    elif lattice == "sc2":
        avec, bmat, tau = _SC_A, _SC_B, np.array([[0, 0, 0], [0.25, 0.25, 0.25]])
        omega = alat ** 3
    else:
        raise ValueError(lattice)
    if nr is None:
        nr = fft_grid_for(alat, avec, 4 * ecut)
    nr = tuple(int(x) for x in nr)
    kf = _rational_vec(kvec)
    kqf = [a + Fraction(b).limit_denominator(1000) for a, b in zip(kf, qvec)]
    k_float = np.array([float(x) for x in kf])
    kq_float = np.array([float(x) for x in kqf])
    mill_k, nl_k, g2_k = sphere(bmat, kf, alat, ecut, nr)
    mill_kq, nl_kq, g2_kq = sphere(bmat, kqf, alat, ecut, nr)
    vrs = gaussian_vloc(rng, nr, bmat, alat)
    tau_cart = tau * alat
    vkb_k, dvan = kb_projectors(rng, _cart(bmat, mill_k, k_float, alat), tau_cart, omega)
    vkb_kq, _ = kb_projectors(np.random.default_rng(0), _cart(bmat, mill_kq, kq_float, alat), tau_cart, omega)
    eig = eigensolver or dense_states
    et, evc = eig(mill_k, nl_k, g2_k, vrs, nr, vkb_k, dvan, nocc)
    if np.array_equal(mill_k, mill_kq) and np.allclose(g2_k, g2_kq):
        evq = evc.copy(order="F")
    else:
        _, evq = eig(mill_kq, nl_kq, g2_kq, vrs, nr, vkb_kq, dvan, nocc)
    alpha_pv = max(2.0 * (et.max() - et.min()), 1e-2)
    # perturbations: the n_pert G with smallest |q+G| (ties by Miller index)
    r = np.arange(-8, 9)
    m = np.stack(np.meshgrid(r, r, r, indexing="ij"), -1).reshape(-1, 3)
    qg = (m @ bmat.astype(np.float64)) + np.array(qvec)[None, :]
    key = np.round((qg * qg).sum(1), 12)
    order = np.lexsort((m[:, 2], m[:, 1], m[:, 0], key))
    gpert = m[order[:n_pert]].astype(np.int32)
    return dict(
        alat=alat, lattice=lattice, ecut=ecut, omega=omega, nr=np.array(nr, dtype=np.int32),
        seed=seed, qvec=np.array(qvec), kvec=np.array(kvec),
        mill_k=mill_k, nl_k=nl_k, g2kin_k=g2_k,
        mill=mill_kq, nl=nl_kq, g2kin=g2_kq, npw=int(mill_kq.shape[0]), npw_k=int(mill_k.shape[0]),
        vrs=vrs, vkb=np.asfortranarray(vkb_kq), dvan=dvan, evc=evc, et=et, evq=evq,
        alpha_pv=alpha_pv, gpert=gpert, nocc=nocc,
    )


def dvbare_box(system, ip):
    """Delta V(r) = exp(i (q+G_p).r), periodic part exp(i G_p.r) on the box (coulomb.f90:129-134)."""
    nr1, nr2, nr3 = [int(x) for x in system["nr"]]
    g = system["gpert"][ip]
    i1 = np.arange(nr1)[None, None, :]
    i2 = np.arange(nr2)[None, :, None]
    i3 = np.arange(nr3)[:, None, None]
    ph = 2 * math.pi * (g[0] * i1 / nr1 + g[1] * i2 / nr2 + g[2] * i3 / nr3)
    return np.exp(1j * ph).reshape(-1)


def freq_imag(nfreq, max_ev):
    """omega = i * linspace(0, max) (configs with imaginary frequencies)."""
    return 1j * np.linspace(0.0, max_ev, nfreq) / RY_EV


def omega_list(freq):
    """solve_linter.f90:237-252: [w, -w(2:)] if w(1)=0 else [w, -w]."""
    freq = np.asarray(freq, dtype=np.complex128)
    if abs(freq[0]) < 1e-14:
        return np.concatenate([freq, -freq[1:]])
    return np.concatenate([freq, -freq])


C3_SYSTEMS = 64
C3_BASE_SEED = 3000


def c3_params(index, base_seed=C3_BASE_SEED):
    """Parameters of system `index` of the uneven batch: simple-cubic cell with 2
    atoms at (0,0,0) and (1/4,1/4,1/4)a, a ~ U[8, 14] bohr, E_cut ~ U[12, 30] Ry,
    bands ~ U{4..32}, perturbations ~ U{1..64}, frequencies ~ U{8..64}; the FFT
    grid is the smooth grid of 4 E_cut kept within 24..48 per axis."""
    rng = np.random.default_rng(base_seed + index)
    a = float(rng.uniform(8.0, 14.0))
    ecut = float(rng.uniform(12.0, 30.0))
    nocc = int(rng.integers(4, 33))
    npert = int(rng.integers(1, 65))
    nfreq = int(rng.integers(8, 65))
    need = fft_grid_for(a, _SC_A, 4 * ecut)[0]
    n = good_fft_size(max(need, 24))
    if n > 48:
        n = 48
    return dict(alat=a, ecut=ecut, nocc=nocc, npert=npert, nfreq=nfreq, nr=(n, n, n), seed=base_seed + index)


def c3_freq(p):
    """Half of the frequencies on the imaginary axis i [0, 60] eV, half on the real
    axis x + 0.1 i eV with x ~ U[-30, 30] eV (sorted); omega_1 = 0."""
    rng = np.random.default_rng(p["seed"] + 100000)
    nf = p["nfreq"]
    ni = nf // 2
    im = 1j * np.linspace(0.0, 60.0, ni) / RY_EV
    re = (np.sort(rng.uniform(-30.0, 30.0, nf - ni)) + 0.1j) / RY_EV
    return np.concatenate([im, re])


def c3_system(index, eigensolver=None, base_seed=C3_BASE_SEED):
    """System `index` of the uneven batch and its frequency list."""
    p = c3_params(index, base_seed)
    s = make_system(p["alat"], "sc2", p["ecut"], p["nocc"], p["seed"], nr=p["nr"], n_pert=p["npert"],
                    eigensolver=eigensolver)
    return s, c3_freq(p)


def config(name: str, seed: int | None = None):
    """The named benchmark systems.  Returns (system, freq)."""
    if name == "c0":
        s = make_system(10.26, "fcc", 15.0, 4, 0 if seed is None else seed, nr=(20, 20, 20), n_pert=1)
        return s, freq_imag(10, 50.0)
    if name == "c4":
        s = make_system(10.26, "fcc", 15.0, 4, 4 if seed is None else seed, nr=(20, 20, 20), n_pert=8)
        return s, freq_imag(16, 50.0)
    if name in ("c1", "c2"):
        s = make_system(10.26, "sc8", 25.0, 16, 1 if seed is None else seed, nr=(40, 40, 40),
                        qvec=(0.05, 0.0, 0.0), n_pert=113)
        rng = np.random.default_rng(101)
        x = np.sort(rng.uniform(-30.0, 30.0, 35))
        return s, (x + 0.1j) / RY_EV
    raise ValueError(name)


def midgap(system):
    """Chemical potential in the gap of the k+q Hamiltonian (where the Green's
    function is evaluated): the midpoint between its nocc-th and (nocc+1)-th
    eigenvalues (dense FP64 eigvalsh; small systems)."""
    nr = [int(v) for v in system["nr"]]
    h = dense_h(system["mill"], system["g2kin"], system["vrs"], nr, system["vkb"], system["dvan"])
    w = np.linalg.eigvalsh(h)
    n = int(system["nocc"])
    return 0.5 * float(w[n - 1] + w[n])
