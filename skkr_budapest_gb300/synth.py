"""Seeded synthetic inputs for the 2D-BZ tau path (host side, numpy).

The reference obtains its inputs from self-consistent potentials (radial
solvers, Madelung, ...), which lie outside the hot path.  The workloads here
replace them with seeded, physically consistent stand-ins:

* complex energies on the reference's semicircle contour (main/zmesh.f:55-83,
  Gauss-Legendre nodes of main/legzero.f);
* IBZ k meshes of main/speck2.f (square lattice, C4v wedge) with the weights
  of main/kmesh2d.f:139-251;
* single-site t-matrices of spherical square wells, in the reference's
  convention t_l = -(1/kappa) sin(delta) exp(i delta) and screened as
  (t - alpha)^-1 (nrsp-scf/tmat.f, rsp-scf/tmat.f:75-92); the screening
  alpha_l is the t-matrix of a repulsive square barrier (main/alphamat.f);
* screened structure constants in real space, G_scr(R) = [G0 (1 - alpha G0)^-1]
  restricted to the central row of a cluster of the first three neighbour
  shells.  This is the lattice-Fourier-transform form of G_scr(k); the
  reference instead evaluates layer-pair Kambe sums per k (main/gstore.f).
* point-group matrices D(g) of C4v in the complex-harmonic lm basis and, for
  the relativistic case, in the (kappa,mu) basis of main/clebsch.f.

Conventions: complex spherical harmonics with the Condon-Shortley phase,
lm index l*l+l+m; free-space structure constants
G0_{LL'}(R) = -4 pi i kappa sum_L'' i^(-l+l'-l'') <Y_L Y*_L' Y_L''> h_l''(kappa R) Y_L''(R),
which expands -exp(i kappa |r-r'|)/(4 pi |r-r'|) between two sites (checked in
tests/test_synth.py).  G(k) = sum_R exp(+i k.R_par) G_scr(R).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

C_LIGHT = 274.072  # rsp-scf/cpacoord_ksave.f:93 (Rydberg units)


# --------------------------------------------------------------------------
# special functions
# --------------------------------------------------------------------------
def _plm_all(lmax: int, x: np.ndarray) -> np.ndarray:
    """Associated Legendre P_l^m(x), m >= 0, Condon-Shortley phase."""
    x = np.asarray(x, float)
    P = np.zeros((lmax + 1, lmax + 1) + x.shape)
    sx = np.sqrt(np.maximum(0.0, 1.0 - x * x))
    P[0, 0] = 1.0
    for m in range(1, lmax + 1):
        P[m, m] = -(2 * m - 1) * sx * P[m - 1, m - 1]
    for m in range(lmax):
        P[m + 1, m] = (2 * m + 1) * x * P[m, m]
    for m in range(lmax + 1):
        for l in range(m + 2, lmax + 1):
            P[l, m] = ((2 * l - 1) * x * P[l - 1, m] - (l + m - 1) * P[l - 2, m]) / (l - m)
    return P


def ylm(lmax: int, v) -> np.ndarray:
    """Complex Y_lm(v) for unit or non-unit vectors v (N,3) -> (N,(lmax+1)^2)."""
    v = np.atleast_2d(np.asarray(v, float))
    r = np.linalg.norm(v, axis=1)
    r = np.where(r == 0.0, 1.0, r)
    ct = np.clip(v[:, 2] / r, -1.0, 1.0)
    ph = np.arctan2(v[:, 1], v[:, 0])
    P = _plm_all(lmax, ct)
    out = np.zeros((len(v), (lmax + 1) ** 2), complex)
    for l in range(lmax + 1):
        for m in range(-l, l + 1):
            am = abs(m)
            nrm = math.sqrt((2 * l + 1) / (4 * math.pi) * math.factorial(l - am) / math.factorial(l + am))
            y = nrm * P[l, am] * np.exp(1j * am * ph)
            if m < 0:
                y = (-1) ** am * np.conj(y)
            out[:, l * l + l + m] = y
    return out


def sph_bessel(lmax: int, x):
    """j_l, n_l, h_l = j_l + i n_l of complex argument (upward recurrence, as main/csbf.f)."""
    x = np.asarray(x, complex)
    j = np.zeros((lmax + 1,) + x.shape, complex)
    n = np.zeros_like(j)
    j[0] = np.sin(x) / x
    n[0] = -np.cos(x) / x
    if lmax >= 1:
        j[1] = np.sin(x) / x ** 2 - np.cos(x) / x
        n[1] = -np.cos(x) / x ** 2 - np.sin(x) / x
    for l in range(2, lmax + 1):
        j[l] = (2 * l - 1) * j[l - 1] / x - j[l - 2]
        n[l] = (2 * l - 1) * n[l - 1] / x - n[l - 2]
    return j, n, j + 1j * n


def hankel1(lmax: int, x):
    """h_l = j_l + i n_l of complex argument by the upward recurrence of h
    itself, h_0 = -i e^{ix}/x, h_-1 = e^{ix}/x: stable for the outgoing wave,
    where j_l + i n_l from their own recurrences cancels once Im x grows
    (relative error 5e-10 at |x| = 18, Im x = 7)."""
    x = np.asarray(x, complex)
    h = np.zeros((lmax + 1,) + x.shape, complex)
    e = np.exp(1j * x) / x
    h[0] = -1j * e
    if lmax >= 1:
        h[1] = h[0] / x - e
    for l in range(1, lmax):
        h[l + 1] = (2 * l + 1) * h[l] / x - h[l - 1]
    return h


def lm_l(lmmax: int) -> np.ndarray:
    return np.array([int(math.isqrt(i)) for i in range(lmmax)])


def _sphere_quadrature(deg: int):
    nq = deg // 2 + 2
    xg, wg = np.polynomial.legendre.leggauss(nq)
    nph = deg + 2
    ph = 2 * math.pi * np.arange(nph) / nph
    ct = np.repeat(xg, nph)
    w = np.repeat(wg, nph) * 2 * math.pi / nph
    phi = np.tile(ph, nq)
    st = np.sqrt(1 - ct * ct)
    return np.stack([st * np.cos(phi), st * np.sin(phi), ct], 1), w


_GAUNT_CACHE: dict = {}


def gaunt_g0(lmax: int) -> np.ndarray:
    """C[L, L', L''] = <Y_L Y*_L' Y_L''> over the sphere, L'' up to 2*lmax."""
    if lmax in _GAUNT_CACHE:
        return _GAUNT_CACHE[lmax]
    l2 = 2 * lmax
    v, w = _sphere_quadrature(2 * lmax + l2 + 2)
    y1 = ylm(lmax, v)
    y3 = ylm(l2, v)
    c = np.einsum("q,qa,qb,qc->abc", w, y1, np.conj(y1), y3)
    c[np.abs(c) < 1e-13] = 0.0
    _GAUNT_CACHE[lmax] = c
    return c


def kappa_of(e: complex) -> complex:
    k = np.sqrt(complex(e))
    return -k if k.imag < 0 else k


def free_g0(e: complex, rvecs: np.ndarray, lmax: int) -> np.ndarray:
    """Free-space structure constants G0_{LL'}(R) for R (N,3) -> (N, LM, LM)."""
    kap = kappa_of(e)
    l2 = 2 * lmax
    lmmax = (lmax + 1) ** 2
    c = gaunt_g0(lmax)
    lv = lm_l(lmmax)
    lv2 = lm_l((l2 + 1) ** 2)
    rvecs = np.atleast_2d(rvecs)
    r = np.linalg.norm(rvecs, axis=1)
    h = hankel1(l2, kap * r)                   # (l2+1, N)
    yr = ylm(l2, rvecs)                        # (N, LM2)
    ph = (1j) ** ((-lv[:, None, None] + lv[None, :, None] - lv2[None, None, :]) % 4)
    coef = -4 * math.pi * 1j * kap * c * ph    # (LM, LM, LM2)
    hy = h[lv2, :].T * yr                      # (N, LM2)
    return np.tensordot(hy, coef, axes=([1], [2]))   # (N, LM, LM), one BLAS product


# --------------------------------------------------------------------------
# contour and k mesh (main/zmesh.f, main/legzero.f, main/speck2.f, main/kmesh2d.f)
# --------------------------------------------------------------------------
def legzero(ng: int):
    """Gauss-Legendre nodes/weights by Newton from the A&S starting values."""
    x = np.zeros(ng)
    w = np.zeros(ng)

    def legpol(xv, l):
        pnm1, pn = 1.0, xv
        for n in range(1, l):
            pnm1, pn = pn, ((2 * n + 1) * xv * pn - n * pnm1) / (n + 1.0)
        return pn, pnm1, l * (xv * pn - pnm1) / (xv * xv - 1.0)

    n = ng // 2
    for i in range(1, n + 1):
        phi = (4 * i - 1) * math.pi / (4 * ng + 2.0)
        xv = math.cos(phi + 1.0 / (8.0 * ng * ng * math.tan(phi)))
        for _ in range(100):
            pl, plm1, dpl = legpol(xv, ng)
            dx = pl / dpl
            xv -= dx
            if abs(dx) <= 1e-14:
                break
        # the weight uses P_{n-1} of the last Newton step, as the reference does
        wv = 2.0 * (1.0 - xv * xv) / (ng * ng * plm1 * plm1)
        x[ng - i], x[i - 1], w[ng - i], w[i - 1] = xv, -xv, wv, wv
    if 2 * n != ng:
        pl, plm1, dpl = legpol(0.0, ng)
        x[n], w[n] = 0.0, 2.0 / (ng * ng * plm1 * plm1)
    return x, w


def zmesh_semicircle(nepanel: int, ebottom: float, etop: float, epsilon: float):
    """Semicircle contour energies and weights (imesh=1, one panel)."""
    x, w = legzero(nepanel)
    r = (etop - ebottom) / 2.0
    z0 = ebottom + r
    if epsilon > 1e-5:
        eps = 1.0 / epsilon
        y1 = -math.log(1.0 + math.pi / eps)
        y2 = 0.0
        y = 0.5 * (y2 - y1) * x + 0.5 * (y2 + y1)
        phi = eps * (np.exp(-y) - 1.0)
        z = r * np.exp(1j * phi) + z0
        ww = -0.5 * (y2 - y1) * eps * np.exp(-y) * 1j * (z - z0) * w
    else:
        phi = 0.5 * (0.0 - math.pi) * x + 0.5 * math.pi
        z = r * np.exp(1j * phi) + z0
        ww = 0.5 * (0.0 - math.pi) * 1j * (z - z0) * w
    return z, ww


def kmesh_square_c4v(nset: int, a2d: float):
    """IBZ of the square lattice (C4v wedge 0 < y <= x < pi/a), weights
    normalised to 1: interior 1, diagonal 1/2 (kmesh2d.f:191-199)."""
    pts = []
    for i in range(1, nset + 1):
        x = 0.5 * (2 * i - 1) / nset
        for j in range(1, i + 1):
            y = 0.5 * (2 * j - 1) / nset
            pts.append((x, y, 0.5 if i == j else 1.0))
    a = np.array(pts)
    xk = a[:, :2] * (math.pi / a2d)
    wk = a[:, 2] / a[:, 2].sum()
    return xk, wk


def kmesh_square_full(nset: int, a2d: float):
    """Full-BZ grid whose C4v-irreducible part is kmesh_square_c4v(nset)."""
    v = (2 * np.arange(1, nset + 1) - 1) / (2.0 * nset)
    v = np.concatenate([-v[::-1], v])
    xx, yy = np.meshgrid(v, v, indexing="ij")
    xk = np.stack([xx.ravel(), yy.ravel()], 1) * (math.pi / a2d)
    return xk, np.full(len(xk), 1.0 / len(xk))


def nk_of_nset(nset: int) -> int:
    return nset * (nset + 1) // 2


# --------------------------------------------------------------------------
# single-site: screening alpha and square-well t-matrices
# --------------------------------------------------------------------------
def _tan_delta(ck, q, r, lmax):
    fb, fn, _ = sph_bessel(lmax + 1, ck * r)
    gb, _, _ = sph_bessel(lmax + 1, q * r)
    l = np.arange(lmax + 1)
    return (ck * fb[l + 1] * gb[l] - q * fb[l] * gb[l + 1]) / (ck * fn[l + 1] * gb[l] - q * fn[l] * gb[l + 1])


def alpha_sqwell(e: complex, vscreen: float, rs: float, lmax: int) -> np.ndarray:
    """main/alphamat.f (iscreen<=1): alpha_l(E) of a barrier vscreen, radius rs."""
    ck = kappa_of(e)
    csk = kappa_of(complex(e) - vscreen)
    tand = _tan_delta(ck, csk, rs, lmax)
    react = -tand / ck
    return react / (1.0 + 1j * ck * react)


def alpha_sqwell_hole(x: complex, vscreen: float, rs: float, lmax: int) -> np.ndarray:
    """Hole screening parameters of skkr_dbogo_bsf main/alphamat.f (holes
    branch): at the energy x = E_F - E (relativistic form x + x^2/c^2, as
    alphamat.f forms it), with the negative square-root branches
    ck = -sqrt(x), csk = -sqrt(x - V), and alpha_h = -react/(1 + i ck react)."""
    ee = complex(x) + complex(x) * complex(x) / (C_LIGHT * C_LIGHT)
    ck = -np.sqrt(ee)
    csk = -np.sqrt(ee - vscreen)
    tand = _tan_delta(ck, csk, rs, lmax)
    react = -tand / ck
    return -react / (1.0 + 1j * ck * react)


def tinv_sqwell_l(e: complex, depth: float, radius: float, lmax: int) -> np.ndarray:
    """Inverse (unscreened) t_l^-1 of an attractive well V=depth<0."""
    ck = kappa_of(e)
    q = kappa_of(complex(e) - depth)
    tand = _tan_delta(ck, q, radius, lmax)
    react = -tand / ck
    t = react / (1.0 + 1j * ck * react)
    return 1.0 / t


def screened_tinv_nonrel(e, depth, radius, alpha, lmax) -> np.ndarray:
    """nrsp-scf/tmat.f: tminv(lm,lm) = tml/(1 - tml*alpha_l), lm-diagonal."""
    tml = tinv_sqwell_l(e, depth, radius, lmax)
    d = tml / (1.0 - tml * alpha)
    lv = lm_l((lmax + 1) ** 2)
    return np.diag(d[lv]).astype(complex)


def pairing_metric(lmax: int) -> np.ndarray:
    """epsilon(kappa mu, kappa -mu) = (-1)^(j-mu): the singlet pairing matrix
    in the (kappa,mu) basis, D epsilon D^T = epsilon for every double-group
    matrix D of the (kappa,mu) representation."""
    lv, kv = kmy_l_kappa(lmax)
    n = len(lv)
    eps = np.zeros((n, n))
    for kap in sorted(set(kv.tolist())):
        a = abs(kap)
        for m in range(-a, a):            # mu = m + 1/2, j = |kappa| - 1/2
            ir = 2 * kap * kap + kap + m       # 0-based index of (kappa, mu)
            irp = 2 * kap * kap + kap - m - 1  # (kappa, -mu)
            if ir < n and irp < n:
                eps[ir, irp] = (-1.0) ** (a - 1 - m)
    return eps


def bdg_tinv(celoc, psq, celoch, psqh, depth, radius, so_split, alpha_e, alpha_h, lmax, delta):
    """Screened BdG t^-1 (4 (lmax+1)^2 square, electron (kappa,mu) block then
    hole block) of a j-split square well.  The physical inverse is
        m = [[t_e^-1(E), delta eps], [delta eps^T, -conj(t_e^-1(E_F - conj E))]]
    (hole t of BdG: t_h(E) = -t_e(-E*)^*, energies relative to E_F; eps the
    singlet pairing metric, so that m is invariant under blockdiag(D, D*), the
    representation under which the electron and the lmtolmconj-transformed
    hole structure constants transform), and the screening of skkr_dbogo_bsf
    rsp-scf/tmat.f subtracts alpha_e / alpha_h on the diagonal of t before
    re-inverting."""
    zero = np.zeros(lmax + 1, complex)
    te = np.diag(screened_tinv_rel(celoc, psq, depth, radius, so_split, zero, lmax))
    th = -np.conj(np.diag(screened_tinv_rel(celoch, psqh, depth, radius, so_split, zero, lmax)))
    km = len(te)
    m = np.zeros((2 * km, 2 * km), complex)
    m[:km, :km] = np.diag(te)
    m[km:, km:] = np.diag(th)
    eps = pairing_metric(lmax)
    m[:km, km:] = delta * eps
    m[km:, :km] = delta * eps.T
    lv, _ = kmy_l_kappa(lmax)
    t = np.linalg.inv(m)
    t[np.arange(km), np.arange(km)] -= np.asarray(alpha_e)[lv]
    t[km + np.arange(km), km + np.arange(km)] -= np.asarray(alpha_h)[lv]
    return np.linalg.inv(t)


def kmy_l_kappa(lmax: int):
    """(l, kappa, mu2) of each (kappa,mu) index of main/clebsch.f, ir = 2k^2+k+mu+1/2."""
    n = 2 * (lmax + 1) ** 2
    lv = np.zeros(n, int)
    kv = np.zeros(n, int)
    for l in range(lmax + 1):
        for kap in ([l] if l > 0 else []) + [-l - 1]:
            j2 = 2 * abs(kap) - 1
            for mu2 in range(-j2, j2 + 1, 2):
                m = (mu2 - 1) // 2
                ir = 2 * kap * kap + kap + m + 1  # 1-based index of (kappa, mu=m+1/2)
                if ir - 1 < n:
                    lv[ir - 1] = l
                    kv[ir - 1] = kap
    return lv, kv


def screened_tinv_rel(e, psq, depth, radius, so_split, alpha, lmax) -> np.ndarray:
    """(kappa,mu)-diagonal screened t^-1 of a square well whose depth is split
    for j = l +- 1/2 by so_split * <l.s> (rsp-scf/tmat.f:75-92 screening)."""
    lv, kv = kmy_l_kappa(lmax)
    ck = kappa_of(psq)
    d = np.zeros(len(lv), complex)
    for i, (l, kap) in enumerate(zip(lv, kv)):
        ls = 0.5 * l if kap < 0 else -0.5 * (l + 1)
        q = kappa_of(complex(psq) - (depth + so_split * ls))
        tand = _tan_delta(ck, q, radius, l)[l]
        react = -tand / ck
        t = react / (1.0 + 1j * ck * react)
        d[i] = 1.0 / (t - alpha[l])
    return np.diag(d)


# --------------------------------------------------------------------------
# single-site radial integrals of the square well (layer DOS inputs)
# --------------------------------------------------------------------------
def _bessel_l_pm(l: int, x):
    """f_{l-1}, f_l, f_{l+1} for f = j and f = n, with j_{-1} = cos x/x, n_{-1} = sin x/x."""
    j, n, _ = sph_bessel(l + 1, x)
    jm = np.cos(x) / x if l == 0 else j[l - 1]
    nm = np.sin(x) / x if l == 0 else n[l - 1]
    return jm, j[l], j[l + 1], nm, n[l], n[l + 1]


def sqwell_fg(p2: complex, vwell: float, radius: float, l: int):
    """Radial integrals F_l = int_0^R Z_l^2 r^2 dr and G_l = int_0^R Z_l J_l r^2 dr
    of a square well V = vwell (r < R) at squared momentum p2, the inputs of the
    layer DOS of nrsp-scf/moment.f:47-110 (lambda = 0) over the well's sphere.

    Normalisation follows the Green function G = Z tau Z - Z J that belongs to
    t = -(1/k) sin(delta) e^{i delta}: outside the well Z_l = j_l(kr) t_l^-1 -
    i k h_l(kr) and J_l = j_l(kr); inside Z_l = A j_l(qr) and J_l = B j_l(qr) +
    C n_l(qr) continue them with matching value and slope at R.  The integrals
    are the closed Lommel forms int t^2 f_l g_l dt = t^3/4 (2 f_l g_l - f_{l-1}
    g_{l+1} - f_{l+1} g_{l-1}); the j_l n_l form tends to (2l+1)/4 at t = 0.
    Products are complex (no conjugation), as in the reference."""
    ck = kappa_of(p2)
    q = kappa_of(complex(p2) - vwell)
    tand = _tan_delta(ck, q, radius, l)[l]
    react = -tand / ck
    t = react / (1.0 + 1j * ck * react)
    xk = ck * radius
    jkm, jk0, _, nkm, nk0, _ = _bessel_l_pm(l, xk)
    x = q * radius
    jm, j0, jp, nm, n0, np_ = _bessel_l_pm(l, x)
    a = (jk0 / t - 1j * ck * (jk0 + 1j * nk0)) / j0
    jr = jk0                                        # J(R)
    djr = ck * (jkm - (l + 1) / xk * jk0)           # J'(R)
    f, df = j0, q * (jm - (l + 1) / x * j0)
    g, dg = n0, q * (nm - (l + 1) / x * n0)
    det = f * dg - df * g                           # = 1 / (q R^2)
    b = (jr * dg - djr * g) / det
    c = (f * djr - df * jr) / det
    ijj = x ** 3 / 2.0 * (j0 * j0 - jm * jp) / q ** 3
    ijn = (x ** 3 / 4.0 * (2.0 * j0 * n0 - jm * np_ - jp * nm) - (2 * l + 1) / 4.0) / q ** 3
    return complex(a * a * ijj), complex(a * (b * ijj + c * ijn))


def sqwell_regular(p2: complex, vwell: float, radius: float, l: int):
    """(a, q) of the regular solution inside the well in sqwell_fg's
    normalisation: Z_l(r) = a j_l(q r) for r < R."""
    ck = kappa_of(p2)
    q = kappa_of(complex(p2) - vwell)
    tand = _tan_delta(ck, q, radius, l)[l]
    react = -tand / ck
    t = react / (1.0 + 1j * ck * react)
    _, jk0, _, _, nk0, _ = _bessel_l_pm(l, ck * radius)
    j0 = _bessel_l_pm(l, q * radius)[1]
    return complex((jk0 / t - 1j * ck * (jk0 + 1j * nk0)) / j0), complex(q)


_GL_NODES = 48


def radial_overlap(za, zb, radius: float, l: int, conj_b: bool = False) -> complex:
    """int_0^R Z_a(r) Z_b(r) r^2 dr of two regular solutions (a, q) of
    sqwell_regular (conj_b: the complex conjugate of Z_b, a hole solution),
    by 48-node Gauss-Legendre quadrature over the sphere: the integrand is
    entire in r, and the upward Bessel recurrence's error near r = 0 meets a
    partner that vanishes like r^l there."""
    x, w = np.polynomial.legendre.leggauss(_GL_NODES)
    r = 0.5 * radius * (x + 1.0)
    wr = 0.5 * radius * w
    fa = za[0] * sph_bessel(l, za[1] * r)[0][l]
    fb = zb[0] * sph_bessel(l, zb[1] * r)[0][l]
    if conj_b:
        fb = np.conj(fb)
    return complex(np.sum(wr * r * r * fa * fb))


def _species_depths(ep, li):
    """Well depths of species A and B of interface layer li (BdG systems have
    one species per layer)."""
    m = ep.meta
    if "depth_a" in m:
        return float(m["depth_a"][li]), float(m["depth_b"][li])
    d = float(m["depth_int"][li])
    return d, d


def bsf_radial(ep):
    """Radial overlaps of the regular solutions that the Bloch spectral
    function of bsf.f contracts with tau (gf.f's Z^R tau Z^L with the
    diagonal, spherical solutions of the square wells of this model):

    F[li, a, b, i] = int Z^a_i Z^b_i r^2 dr, a and b over species A, B (the
    right solution of species a, the left of species b), i the basis index:
    lm (non-relativistic), (kappa,mu) of the j-split well (relativistic,
    momentum psq, large component), or for BdG the electron block (psq) then
    the hole block (hole solutions: the conjugates of the electron ones at
    the hole momentum psqh, the pairing living in t^-1).

    Feh[li, a, b, j, i] (BdG only, else None) = int Z^{e,a}_j Z^{h,b}_i r^2 dr
    for electron index j and hole index i of the same l, zero otherwise: the
    electron-hole block that the anomalous components contract."""
    lmax = ep.lmax
    radius, so = ep.meta["radius"], ep.meta.get("so_split", 0.0)
    bdg = ep.irel == 2
    nde = ep.lkmax // 2 if bdg else ep.lkmax
    if ep.irel:
        lv, kv = kmy_l_kappa(lmax)
    else:
        lv, kv = lm_l(nde), None
    lv = np.asarray(lv)[:nde]
    F = np.zeros((ep.nintfc, 2, 2, ep.lkmax), complex)
    Feh = np.zeros((ep.nintfc, 2, 2, nde, nde), complex) if bdg else None
    psqh = ep.meta.get("psqh")

    def wells(depth):
        zs, zh = [], []
        for i in range(nde):
            l = int(lv[i])
            v = depth
            if kv is not None:
                kap = int(kv[i])
                v += so * (0.5 * l if kap < 0 else -0.5 * (l + 1))
            zs.append((l, sqwell_regular(ep.psq, v, radius, l)))
            if bdg:
                zh.append((l, sqwell_regular(psqh, v, radius, l)))
        return zs, zh

    for li in range(ep.nintfc):
        sp = [wells(d) for d in _species_depths(ep, li)]
        for a in range(2):
            for b in range(2):
                ea, ha = sp[a]
                eb, hb = sp[b]
                cache = {}
                for i in range(nde):
                    l = ea[i][0]
                    key = (l, ea[i][1], eb[i][1])
                    if key not in cache:
                        cache[key] = radial_overlap(ea[i][1], eb[i][1], radius, l)
                    F[li, a, b, i] = cache[key]
                    if bdg:
                        # both hole solutions conjugated: the conjugate overlap
                        F[li, a, b, nde + i] = np.conj(radial_overlap(ha[i][1], hb[i][1], radius, l))
                if bdg:
                    for j in range(nde):
                        for i in range(nde):
                            if ea[j][0] == ha[i][0]:
                                key = ("eh", ea[j][0], ea[j][1], hb[i][1])
                                if key not in cache:
                                    cache[key] = radial_overlap(ea[j][1], hb[i][1], radius, ea[j][0], conj_b=True)
                                Feh[li, a, b, j, i] = cache[key]
    return F, Feh


def _lms_pairs(lmax: int):
    """(lm, lm', m) of the lm pairs with l = l' and m = -m' (the selection of
    skkr_dbogo_bsf/rsp-scf/pairing.f:46-200), lm in the order l = 0..lmax,
    m = -l..l."""
    out = []
    lm = 0
    for l in range(lmax + 1):
        for m in range(-l, l + 1):
            out.append((lm, lm - 2 * m, m))
            lm += 1
    return out


def pairing_kmy(lmax: int) -> dict:
    """The four pairing operators of rsp-scf/pairing.f:46-200 in the (kappa,mu)
    basis: singlet (i sigma_y), triplet with unequal spins (T0), and the
    equal-spin triplets (up, down), each built in the (l, m, s)
    representation on l = l', m = -m' and taken to (kappa,mu) with the
    Clebsch-Gordan matrix as rsp-scf/matlms.f:93-126 (matkmy) does (U^T X U, no
    conjugation; spin index 1 of the reference pairs with u1)."""
    lmmax = (lmax + 1) ** 2
    U = clebsch_u(lmax)
    out = {}
    for name in ("singlet", "t0", "tup", "tdown"):
        X = np.zeros((2 * lmmax, 2 * lmmax), complex)
        for lm, lmp, m in _lms_pairs(lmax):
            sm, smp = (-1.0) ** m, (-1.0) ** (-m)
            if name == "singlet":
                X[lm, lmmax + lmp] = 0.5 * sm
                X[lmmax + lm, lmp] = -0.5 * sm
            elif name == "t0":
                X[lm, lmmax + lmp] = 0.5 * smp
                X[lmmax + lm, lmp] = 0.5 * smp
            elif name == "tup":
                X[lm, lmp] = 0.5 * smp
                X[lmmax + lm, lmmax + lmp] = -0.5 * smp
            else:
                X[lm, lmp] = -0.5j * smp
                X[lmmax + lm, lmmax + lmp] = -0.5j * smp
        out[name] = U.T @ X @ U
    return out


def layer_dos_inputs(ep, which: str = "a"):
    """Per-basis-index F, G (nintfc, lk) of the interface layers of an
    EnergyProblem for species `which` ('a' or 'b'): lm-resolved F_l, G_l
    (non-relativistic) or (kappa,mu)-resolved F_kappa, G_kappa of the j-split
    well (relativistic, momentum psq, large component only)."""
    depths = ep.meta["depth_" + which]
    radius, so = ep.meta["radius"], ep.meta["so_split"]
    lk = ep.lkmax
    F = np.zeros((ep.nintfc, lk), complex)
    G = np.zeros_like(F)
    if ep.irel:
        lv, kv = kmy_l_kappa(ep.lmax)
    else:
        lv = lm_l(lk)
        kv = None
    for li in range(ep.nintfc):
        cache = {}
        for i in range(lk):
            l = int(lv[i])
            if kv is None:
                key, v = l, depths[li]
            else:
                kap = int(kv[i])
                ls = 0.5 * l if kap < 0 else -0.5 * (l + 1)
                key, v = kap, depths[li] + so * ls
            if key not in cache:
                cache[key] = sqwell_fg(ep.psq, v, radius, l)
            F[li, i], G[li, i] = cache[key]
    return F, G


# --------------------------------------------------------------------------
# lattice, cluster and real-space screened structure constants
# --------------------------------------------------------------------------
@dataclass
class Stacking:
    """A Bravais stacking of identical square layers, ABAB with (1/2,1/2) shift."""
    a2d: float      # in-plane square lattice constant
    dz: float       # interlayer spacing
    name: str = ""

    def site(self, n: int, i: int, j: int) -> np.ndarray:
        s = 0.5 * (n % 2)
        return np.array([(i + s) * self.a2d, (j + s) * self.a2d, n * self.dz])


def fcc001(a: float) -> Stacking:
    return Stacking(a / math.sqrt(2.0), a / 2.0, "fcc(001)")


def bcc001(a: float) -> Stacking:
    return Stacking(a, a / 2.0, "bcc(001)")


_CLUSTERS = {}


def cluster(st: Stacking, nshell: int = 3):
    """Sites within the first nshell neighbour shells of the origin (with it).
    Returns (vectors (N,3), layer offsets (N,), nn distance).  The geometry
    does not depend on the energy: it is computed once per stacking."""
    key = (st.a2d, st.dz, nshell)
    if key not in _CLUSTERS:
        _CLUSTERS[key] = _cluster(st, nshell)
    v, n, d = _CLUSTERS[key]
    return v.copy(), n.copy(), d


def _cluster(st: Stacking, nshell: int):
    vs, ns = [], []
    rng = range(-6, 7)
    for n in range(-6, 7):
        for i in rng:
            for j in rng:
                v = st.site(n, i, j) - st.site(0, 0, 0)
                vs.append(v)
                ns.append(n)
    vs = np.array(vs)
    ns = np.array(ns)
    d = np.round(np.linalg.norm(vs, axis=1), 8)
    shells = np.unique(d)
    cut = shells[nshell] + 1e-6
    sel = d <= cut
    order = np.lexsort((vs[sel][:, 1], vs[sel][:, 0], d[sel]))
    return vs[sel][order], ns[sel][order], shells[1]


def lm_conj_matrix(lmax: int) -> np.ndarray:
    """T of main/relmtrx.f lmtolmconj (skkr_dbogo_bsf): |lm> -> |lm>*, T(lm, l -m) = (-1)^m;
    T is its own inverse."""
    lmmax = (lmax + 1) ** 2
    t = np.zeros((lmmax, lmmax))
    for l in range(lmax + 1):
        for m in range(-l, l + 1):
            t[l * l + l + m, l * l + l - m] = (-1.0) ** m
    return t


def screened_realspace(e_struct: complex, vecs: np.ndarray, alpha: np.ndarray, lmax: int,
                       hole: bool = False) -> np.ndarray:
    """Central row of G_scr = (1 - G0 alpha)^-1 G0 on the cluster `vecs`
    (vecs[0] must be the origin).  Returns (N, LM, LM): G_scr(0 -> R_n).
    hole=True screens the hole structure constants of skkr_dbogo_bsf
    main/gstore.f:208-216, G0_h(n, m) = -T G0(m, n)^dagger T, with the hole alpha."""
    lmmax = (lmax + 1) ** 2
    nsite = len(vecs)
    lv = lm_l(lmmax)
    al = np.asarray(alpha)[lv]
    big = np.zeros((nsite * lmmax, nsite * lmmax), complex)
    pair_n, pair_m = np.nonzero(~np.eye(nsite, dtype=bool))
    g = free_g0(e_struct, vecs[pair_n] - vecs[pair_m], lmax)
    big.reshape(nsite, lmmax, nsite, lmmax)[pair_n, :, pair_m, :] = g
    if hole:
        tm = np.kron(np.eye(nsite), lm_conj_matrix(lmax))
        big = -tm @ big.conj().T @ tm
    # (1 - G0 alpha) X = G0, alpha diagonal per site; only the central rows of
    # X are kept, so the rows of (1 - G0 alpha)^-1 come from lmmax solves of the
    # transposed system
    amat = np.eye(nsite * lmmax, dtype=complex) - big * np.tile(al, nsite)[None, :]
    rinv = np.linalg.solve(amat.T, np.eye(nsite * lmmax, lmmax, dtype=complex)).T   # (lmmax, N)
    row = (rinv @ big).reshape(lmmax, nsite, lmmax).transpose(1, 0, 2)
    # G_scr(0 -> R_n) couples site 0 (row) to site n (column): G_{0n}
    return np.ascontiguousarray(row)


@dataclass
class RTable:
    """Real-space screened table grouped by structure-constant block."""
    lmax: int
    nblk: int
    rstart: np.ndarray     # int32 (nblk+1)
    rvec: np.ndarray       # float64 (nR, 2) in-plane displacement
    gR: np.ndarray         # complex128 (nR, LM, LM), element [r, a, b] = G_ab
    jmax: int
    blk_of_j: dict = field(default_factory=dict)


def build_rtable(st: Stacking, e_struct: complex, alpha: np.ndarray, lmax: int, nshell: int = 3,
                 hole: bool = False, nshell_screen: int | None = None) -> RTable:
    """Screened table of the first nshell neighbour shells; the screening
    inversion runs on the larger cluster of nshell_screen shells (default:
    the same) so that the kept couplings do not see the cluster boundary."""
    big, nsb, _ = cluster(st, nshell_screen or nshell)
    vecs, ns, _ = cluster(st, nshell)
    gbig = screened_realspace(e_struct, big, alpha, lmax, hole)
    g = gbig[:len(vecs)]            # cluster() orders sites by distance: inner shells first
    assert np.allclose(big[:len(vecs)], vecs)
    jmax = int(np.max(np.abs(ns)))
    starts, rv, gr, blk_of_j = [0], [], [], {}
    for j in range(-jmax, jmax + 1):
        sel = np.nonzero(ns == j)[0]
        if len(sel) == 0:
            continue
        blk_of_j[j] = len(starts) - 1
        rv.append(vecs[sel, :2])
        gr.append(g[sel])
        starts.append(starts[-1] + len(sel))
    return RTable(lmax, len(starts) - 1, np.array(starts, np.int32), np.concatenate(rv),
                  np.concatenate(gr), jmax, blk_of_j)


def blkmap_translation_invariant(rt: RTable, nslot: int, mi: int) -> np.ndarray:
    """blkmap[slot][i][j+jmax] for a stacking where every layer is equivalent."""
    nj = 2 * rt.jmax + 1
    m = -np.ones((nslot, mi, nj), np.int32)
    for j, b in rt.blk_of_j.items():
        m[:, :, j + rt.jmax] = b
    return m


def gk_blocks(rt: RTable, k: np.ndarray) -> np.ndarray:
    """numpy G(k) blocks (nblk, LM, LM) -- used by the synthetic checks only."""
    ph = np.exp(1j * (rt.rvec @ np.asarray(k, float)))
    out = np.zeros((rt.nblk,) + rt.gR.shape[1:], complex)
    for b in range(rt.nblk):
        s, e = rt.rstart[b], rt.rstart[b + 1]
        out[b] = np.einsum("r,rab->ab", ph[s:e], rt.gR[s:e])
    return out


# --------------------------------------------------------------------------
# point group C4v: lm and (kappa,mu) representations
# --------------------------------------------------------------------------
def c4v_ops():
    """3x3 matrices of C4v about z (E, C4, C2, C4^3, sx, sy, sd, sd')."""
    def rz(t):
        c, s = round(math.cos(t)), round(math.sin(t))
        return np.array([[c, -s, 0], [s, c, 0], [0, 0, 1]], float)
    ops = [rz(0), rz(math.pi / 2), rz(math.pi), rz(3 * math.pi / 2)]
    ops += [np.diag([-1.0, 1, 1]), np.diag([1.0, -1, 1]),
            np.array([[0, 1, 0], [1, 0, 0], [0, 0, 1]], float),
            np.array([[0, -1, 0], [-1, 0, 0], [0, 0, 1]], float)]
    return ops


def d_orbital(op: np.ndarray, lmax: int) -> np.ndarray:
    """D_{L'L}(g) with Y_L(g^-1 r) = sum_L' Y_L'(r) D_{L'L}(g)."""
    v, w = _sphere_quadrature(4 * lmax + 4)
    y = ylm(lmax, v)
    yg = ylm(lmax, v @ op)   # rows: (g^-1 v)^T = v^T g for orthogonal g
    return np.einsum("q,qa,qb->ab", w, np.conj(y), yg)


def _su2(op: np.ndarray) -> np.ndarray:
    """Spin-1/2 matrix of the proper part of op, basis (up, down)."""
    r = op * np.linalg.det(op)
    ang = math.acos(max(-1.0, min(1.0, (np.trace(r) - 1) / 2)))
    if abs(ang) < 1e-12:
        return np.eye(2, dtype=complex)
    if abs(ang - math.pi) < 1e-9:
        axis = np.sqrt(np.maximum(0.0, (np.diag(r) + 1) / 2))
        i0 = int(np.argmax(axis))
        for k in range(3):
            if k != i0 and r[i0, k] < 0:
                axis[k] = -axis[k]
    else:
        axis = np.array([r[2, 1] - r[1, 2], r[0, 2] - r[2, 0], r[1, 0] - r[0, 1]]) / (2 * math.sin(ang))
    sx = np.array([[0, 1], [1, 0]], complex)
    sy = np.array([[0, -1j], [1j, 0]], complex)
    sz = np.array([[1, 0], [0, -1]], complex)
    ns = axis[0] * sx + axis[1] * sy + axis[2] * sz
    return math.cos(ang / 2) * np.eye(2) - 1j * math.sin(ang / 2) * ns


def clebsch_u(lmax: int) -> np.ndarray:
    """U[(s, lm), kmy] mapping (lm x spin) to (kappa,mu) as main/clebsch.f:
    |kmy> = u1 |lm=ind1, s=-1/2> + u2 |lm=ind2, s=+1/2>; row index s*LM + lm
    with s=0 for spin down, 1 for spin up."""
    lmmax = (lmax + 1) ** 2
    n = 2 * lmmax
    u1 = np.zeros(72)
    u2 = np.zeros(72)
    i1 = np.zeros(72, int)
    i2 = np.zeros(72, int)
    inr = 0
    for l in range(6):
        tl = 2 * l + 1.0
        for m in range(-l, l + 1):
            inr += 1
            kap = l
            if kap != 0:
                ir = 2 * kap * kap + kap + m
                u1[ir - 1], i1[ir - 1] = math.sqrt((l + m) / tl), inr
                ir += 1
                u2[ir - 1], i2[ir - 1] = -math.sqrt((l - m) / tl), inr
            kap = -l - 1
            ir = 2 * kap * kap + kap + m
            u1[ir - 1], i1[ir - 1] = math.sqrt((l - m + 1) / tl), inr
            ir += 1
            u2[ir - 1], i2[ir - 1] = math.sqrt((l + m + 1) / tl), inr
    i1[i1 == 0] = 1
    i2[i2 == 0] = 1
    U = np.zeros((2 * lmmax, n))
    for k in range(n):
        U[0 * lmmax + i1[k] - 1, k] += u1[k]
        U[1 * lmmax + i2[k] - 1, k] += u2[k]
    return U


def d_relativistic(op: np.ndarray, lmax: int) -> np.ndarray:
    lmmax = (lmax + 1) ** 2
    do = d_orbital(op, lmax)
    s = _su2(op)                      # (up, down)
    sd = s[::-1, ::-1]                # reorder to (down, up)
    full = np.kron(sd, do)            # row index s*LM + lm
    U = clebsch_u(lmax)
    return U.T @ full @ U


def point_group_mats(lmax: int, irel: int):
    """L_g = D(g), R_g = D(g)^dagger for the C4v operations."""
    ops = c4v_ops()
    if irel:
        ds = [d_relativistic(o, lmax) for o in ops]
    else:
        ds = [d_orbital(o, lmax) for o in ops]
    lg = np.array(ds)
    rg = np.conj(np.transpose(lg, (0, 2, 1)))
    return lg, rg
