"""Reference-faithful k-space structure constants of a stack of 2D lattices
(test infrastructure: the oracle, never the product path).

The reference does not Fourier-transform a real-space table: per k point it
evaluates the 2D lattice sums of the layer-pair structure constants with
Kambe's Ewald split (main/gstore.f:6-283 calling main/kamstr.f:20-392) and
screens them on a finite slab in k space, G' = G (1 - alpha G)^-1
(main/scrstr.f:2-138).  This module restates those routines in numpy so that
the G_scr(k) the GPU path builds from its real-space table can be set beside
the reference's formulation:

  cerf      main/cerf.f        the Faddeeva function w(z) = exp(-z^2) erfc(-iz)
                               (scipy.special.wofz stands in for the series /
                               continued-fraction evaluation of cerf.f)
  incgamma  main/incgamma.f:7  Gamma(1/2 - n, z) by downward recursion from erfc
  ilkam     main/ilkam.f:5     the real-space Ewald integrals I_l
  delkam    main/delkam.f:5    the Delta_n integrals of the out-of-plane case
  ylmc      main/ylmc.f        complex Y_lm, Condon-Shortley phase, from its
                               power-series table of d^m P_l / dx^m
  blm       main/blm.f         Gaunt integral of three Y_lm
  gauntcalc main/gauntcalc.f:2 the coupling table of kamstr
  kamstr    main/kamstr.f:20   D_L = reciprocal part (formulas 35 / 50 of the
                               code's comments) + real-space part (formula 47)
                               + the s = 0 correction (formula 55), then
                               alm = sum_L gau D_L

  sphrm     main/sphrm.f       Y_lm of complex angles (evanescent waves)
  directg   main/directg.f:2   the plane-wave form of the same lattice sum,
                               which gstore.f:158-166 uses for layer pairs
                               with |s_z| |b|_min >= 5
  gstore_block                 that choice between kamstr and directg
  screened_slab                gstore.f:146-185 + scrstr.f: the slab of layers
                               and its screening in k space

Lattice vectors are taken within fixed cut-offs (`gcut`, `rcut`) instead of
the shell-by-shell stopping rules of kamstr.f (1e-10 absolute change) and
directg.f (1e-12 relative), which only decide where a converged sum is
truncated."""
from __future__ import annotations

import math

import numpy as np
from scipy.special import wofz

CI = 1j
CTOL = 1.0e-4          # main/kamstr.f: 'parameter (ctol=1.d-4)'


def cerf(z):
    return wofz(z)


def _fac(n):
    return float(math.factorial(n))


def incgamma(n: int, z: complex) -> np.ndarray:
    """main/incgamma.f:7-48 (n >= 0): gam[i] = Gamma(1/2 - i, z), i = 0..n."""
    gam = np.zeros(n + 1, complex)
    ex = np.exp(-z)
    sz = np.sqrt(z)
    a = sz * np.exp(CI * math.pi / 2.0)
    s = math.sqrt(math.pi) * ex * cerf(a)
    gam[0] = s
    b = 0.5 - 1.0
    zb = sz
    for i in range(1, n + 1):
        zb = zb / z
        s = (s - zb * ex) / b
        gam[i] = s
        b -= 1.0
    return gam


def ilkam(l: int, alpha: complex, t: float, kappa: complex) -> np.ndarray:
    """main/ilkam.f:5-56: the real-space integrals delta(0..l) at distance t."""
    delta = np.zeros(l + 1, complex)
    z = kappa * t
    x = alpha
    sx = np.sqrt(x)
    b = 2.0 / z
    dc = math.sqrt(math.pi) / 2.0
    a = z / 2.0 / sx
    ex = np.exp(x - a * a)
    c = CI * a
    ap = sx + c
    am = -sx + c
    wp = cerf(ap)
    wm = cerf(am)
    c = ex * dc
    dl = (wp + wm) * c * b
    delm1 = (wp - wm) * c / CI
    delta[0] = dl
    b = b * b
    cx = sx
    d = 0.5
    for i in range(1, l + 1):
        cx = cx / x
        del2 = (d * dl - delm1 + cx * ex) * b
        delta[i] = del2
        delm1 = dl
        dl = del2
        d += 1.0
    return delta


def delkam(n: int, x: complex, zz: complex) -> np.ndarray:
    """main/delkam.f:5-57: delta(0..n) of the out-of-plane reciprocal term."""
    delta = np.zeros(max(n, 1) + 1, complex)
    z = np.sqrt(zz)
    sx = np.sqrt(x)
    dc = math.sqrt(math.pi) / 2.0
    b = 2.0 / z
    a = z / 2.0 / sx
    ex = np.exp(a * a - x)
    c = CI * sx
    am = -a + c
    ap = a + c
    wm = cerf(am)
    wp = cerf(ap)
    c = ex * dc
    delta[0] = (wm + wp) * c
    delta[1] = (wm - wp) * c * b * CI
    fc = sx
    b = b * b
    d = 0.5
    for i in range(0, n - 1):
        fc = fc / x
        delta[i + 2] = b * (-d * delta[i + 1] - delta[i] + ex * fc)
        d += 1.0
    return delta[:n + 1]


_YLM_B: dict = {}


def _ylm_table(lmax: int) -> np.ndarray:
    """b[l, m, k] of main/ylmc.f: the power-series coefficients of
    d^m P_l / dx^m, from the coefficients a[l, n] of P_l (its recursion
    a(l,n) = (2l-1)/l a(l-1,n-1) - (l-1)/l a(l-2,n)) and n!/(n-m)!."""
    if lmax in _YLM_B:
        return _YLM_B[lmax]
    L = max(lmax, 2)
    a = np.zeros((L + 1, L + 1))
    a[0, 0], a[1, 1], a[2, 0], a[2, 2] = 1.0, 1.0, -0.5, 1.5
    for l in range(3, L + 1):
        fa1, fa2 = (2 * l - 1) / l, -(l - 1) / l
        a[l, 0] = fa2 * a[l - 2, 0]
        for n in range(1, l - 1):
            a[l, n] = fa1 * a[l - 1, n - 1] + fa2 * a[l - 2, n]
        a[l, l - 1] = fa1 * a[l - 1, l - 2]
        a[l, l] = fa1 * a[l - 1, l - 1]
    f = np.zeros((L + 1, L + 1))
    for n in range(L + 1):
        f[n, 0] = 1.0
        for m in range(n):
            f[n, m + 1] = f[n, m] * (n - m)
    b = np.zeros((L + 1, L + 1, L + 1))
    for l in range(L + 1):
        for m in range(l + 1):
            for k in range(l - m + 1):
                b[l, m, k] = a[l, k + m] * f[k + m, m]
    _YLM_B[lmax] = b
    return b


def ylmc(v, lmax: int) -> np.ndarray:
    """main/ylmc.f: complex Y_lm(v), index l(l+1)+m, Condon-Shortley phase."""
    x, y, z = (float(t) for t in v)
    r = math.sqrt(x * x + y * y + z * z)
    if r < 1e-16:
        cth, ephi = 0.0, 1.0 + 0j
    else:
        cth = z / r
        d = math.sqrt(x * x + y * y)
        ephi = 1.0 + 0j if d < 1e-6 else (x + CI * y) / d
    px = math.sqrt(max(1.0 - cth * cth, 0.0)) + 1e-30
    b = _ylm_table(lmax)
    p = cth ** np.arange(lmax + 1)
    out = np.zeros((lmax + 1) ** 2, complex)
    for l in range(lmax + 1):
        for m in range(-l, l + 1):
            mb = abs(m)
            cf = math.sqrt((2 * l + 1) * _fac(l - mb) / (4 * math.pi * _fac(l + mb))) * CI ** (m + mb)
            t = float(b[l, mb, :l + 1] @ p[:l + 1])
            out[l * (l + 1) + m] = cf * px ** mb * t * ephi ** m
    return out


def _facr(n, m):
    # main/fac.f: n! / (n - m)!
    f = 1.0
    for i in range(n - m + 1, n + 1):
        f *= float(i)
    return f


def blm(il1, im1, il2, im2, il3, im3) -> float:
    """main/blm.f: the Gaunt integral of Y_l1m1 Y_l2m2 Y_l3m3 over the sphere."""
    l1, l2, l3 = il1, il2, il3
    m1, m2, m3 = abs(im1), abs(im2), abs(im3)
    if abs(im1 + im2 + im3) + (l1 + l2 + l3) % 2 != 0 or l1 > l2 + l3 or l1 < abs(l2 - l3):
        return 0.0
    l, m = l1, m1
    m1 = max(m1, m2, m3)
    if m1 != m:
        if m1 == m2:
            l1, l2, m2 = l2, l, m
        else:
            l1, l3, m3 = l3, l, m
    if l2 < l3:
        l, m = l2, m2
        l2, m2 = l3, m3
        l3, m3 = l, m
    is_ = (l1 + l2 + l3) // 2
    sgn = 1 if l3 - m1 >= 0 else -1
    b = ((-1.0) ** (is_ - l2 - m3 + m1) * math.sqrt((2 * l1 + 1) * (2 * l2 + 1) * (2 * l3 + 1) / math.pi)
         / (2 * (2 * is_ + 1)) * math.sqrt(_facr(l1 + m1, m1 + m1)) / _facr(is_ - l1, is_ - l1)
         * math.sqrt(_facr(l2 + m2, m2 + m2)) / _facr(is_ - l2, is_ - l2) * math.sqrt(_facr(l3 + m3, m3 + m3))
         * _facr(max(l2 + l3 - m1, l2 - l3 + m1), abs(2 * (l3 - m1))) ** sgn)
    if l3 == 0:
        return b
    for i in range(1, l3 + 1):
        b /= 2 * (2 * (is_ - i) + 1)
    a = aa = 1.0
    i1, i2, i3, i4, i5, i6 = l1 + m1, max(1, l2 + l3 - m1), 0, l1 - m1, l2 - l3 + m1, l3 - m3
    it = min(i4, i6)
    if it == 0:
        return b
    for _ in range(it):
        i1 += 1
        i3 += 1
        i5 += 1
        aa = -aa * i1 * i4 * i6 / (i2 * i3 * i5)
        a += aa
        i2 -= 1
        i4 -= 1
        i6 -= 1
    return a * b


_GAU: dict = {}


def gauntcalc(lmax: int) -> np.ndarray:
    """main/gauntcalc.f:2-28 as an array gau[lm1, lm2, lm] (lm up to 2 lmax)."""
    if lmax in _GAU:
        return _GAU[lmax]
    nl, nl2 = (lmax + 1) ** 2, (2 * lmax + 1) ** 2
    gau = np.zeros((nl, nl, nl2))
    for l1 in range(lmax + 1):
        for m1 in range(-l1, l1 + 1):
            for l2 in range(lmax + 1):
                for m2 in range(-l2, l2 + 1):
                    for l in range(2 * lmax + 1):
                        for m in range(-l, l + 1):
                            e = -l2 - l + l1 + 2 * m1
                            v = blm(l2, m2, l1, -m1, l, m)
                            if v != 0.0:
                                gau[l1 * (l1 + 1) + m1, l2 * (l2 + 1) + m2, l * (l + 1) + m] = \
                                    v * 4.0 * math.pi * (-1.0) ** (e // 2)
    _GAU[lmax] = gau
    return gau


class Lattice2D:
    """Direct and reciprocal vectors of a 2D Bravais lattice (a1, a2 in a.u.)."""

    def __init__(self, a1, a2):
        self.a1 = np.asarray(a1, float)
        self.a2 = np.asarray(a2, float)
        self.area = abs(self.a1[0] * self.a2[1] - self.a1[1] * self.a2[0])
        rot = np.array([[0.0, 1.0], [-1.0, 0.0]])
        self.b1 = 2 * math.pi * (rot @ self.a2) / (self.a1 @ (rot @ self.a2))
        self.b2 = 2 * math.pi * (rot @ self.a1) / (self.a2 @ (rot @ self.a1))
        self.bmin = min(np.linalg.norm(self.b1), np.linalg.norm(self.b2))

    @staticmethod
    def _points(u, v, cut, centre=(0.0, 0.0)):
        n = int(cut / min(np.linalg.norm(u), np.linalg.norm(v)) * 1.5) + 3
        i, j = np.meshgrid(np.arange(-n, n + 1), np.arange(-n, n + 1), indexing="ij")
        p = i.ravel()[:, None] * u + j.ravel()[:, None] * v
        d = np.linalg.norm(p - np.asarray(centre), axis=1)
        return p[d <= cut]

    def rvecs(self, cut, centre=(0.0, 0.0)):
        return self._points(self.a1, self.a2, cut, centre)

    def gvecs(self, cut, centre=(0.0, 0.0)):
        return self._points(self.b1, self.b2, cut, centre)


def kambe_dlm(e: complex, kx: float, ky: float, sep, lmax2: int, lat: Lattice2D, factor: float = 1.0,
              gcut: float = 12.0, rcut: float = 40.0) -> np.ndarray:
    """main/kamstr.f:72-355: the lattice sums D_L(k, s), L up to lmax2, of
    kamstr (dlm1 + dlm2) for the separation sep = (sx, sy, sz)."""
    lmmx = (lmax2 + 1) ** 2
    kappa = np.sqrt(complex(e))
    v2 = lat.area
    cs1 = -1.0 / v2 / kappa
    cs2 = -kappa / 2.0 / math.sqrt(math.pi)
    alpha = factor * e * v2 / 4.0 / math.pi
    w = alpha * 2.0 / e
    fac = [_fac(i) for i in range(2 * lmax2 + 1)]
    # F(lm) of kamstr.f:84-95: 2^-l sqrt((2l+1)(l+m)!(l-m)!)
    flm = np.zeros(lmmx)
    for l in range(lmax2 + 1):
        for m in range(l + 1):
            a = 2.0 ** (-l) * math.sqrt((2 * l + 1) * fac[l + m] * fac[l - m])
            flm[l * (l + 1) + m] = a
            flm[l * (l + 1) - m] = a
    # formula 55 (kamstr.f:121-124)
    a = np.sqrt(alpha)
    c = CI * (np.exp(-alpha) - cerf(a)) - 1.0 / math.sqrt(math.pi) / a
    d003 = -kappa * (np.exp(alpha) * c - CI) / 2.0 / math.sqrt(math.pi)
    sx, sy, sz = (float(t) for t in sep)
    s = math.sqrt(sx * sx + sy * sy + sz * sz)
    dlm1 = np.zeros(lmmx, complex)
    dlm2 = np.zeros(lmmx, complex)
    if s < CTOL:
        dlm1[0] += d003
    if s > CTOL and abs(sz) < CTOL:   # kamstr.f:136-140: in-plane pairs get sz = 1.1 ctol
        sz = 1.1 * CTOL
        s = math.sqrt(sx * sx + sy * sy + sz * sz)
    f35 = s > CTOL and abs(sz) > CTOL
    cs = (kappa * sz) ** np.arange(lmax2 + 1)
    # reciprocal-space part (formulas 35 and 50)
    for g in lat.gvecs(gcut, centre=(-kx, -ky)):
        gkx, gky = g[0] + kx, g[1] + ky
        km2 = gkx * gkx + gky * gky
        kp = np.sqrt(e - km2)
        km = math.sqrt(km2)
        ex2 = (gkx + CI * gky) / km if km > 1e-10 else 1.0 + 0j
        xc = np.exp(-CI * math.pi) * (e - km * km) * w / 2.0
        gam = incgamma(lmax2, xc)
        cp = (kp / kappa) ** (2 * np.arange(lmax2 + 1) - 1)
        cm = (km / kappa) ** np.arange(lmax2 + 1)
        if f35:
            dl = delkam(lmax2, xc, (kp * sz) ** 2)
            ex1 = np.exp(CI * (gkx * sx + gky * sy)) * cs1
            for l in range(lmax2 + 1):
                for m in range(-l, l + 1):
                    mm = abs(m)
                    ex = ex2 ** (-m) * ex1
                    ipar = (l - mm) % 2
                    csum = 0j
                    for n in range(l - mm + 1):
                        b = 0j
                        for k in range(n + (n + ipar) % 2, min(2 * n, l - mm) + 1, 2):
                            i, j = 2 * n - k, l - k
                            cc = cs[i] * cm[j] / fac[i] / fac[k - n]
                            b += cc / fac[(l - mm - k) // 2] / fac[(l + mm - k) // 2]
                        csum += cp[n] * dl[n] * b
                    dlm1[l * (l + 1) + m] += ex * flm[l * (l + 1) + m] * csum * CI ** (1 - m)
        else:
            for l in range(lmax2 + 1):
                for m in range(-l, l + 1):
                    mm = abs(m)
                    if (l - mm) % 2:
                        continue
                    ex = ex2 ** (-m) * cs1
                    csum = 0j
                    for n in range((l - mm) // 2 + 1):
                        csum += (cp[n] * cm[l - 2 * n] / fac[n] * gam[n]
                                 / fac[(l - mm - 2 * n) // 2] / fac[(l + mm - 2 * n) // 2])
                    dlm1[l * (l + 1) + m] += ex * csum * flm[l * (l + 1) + m] * CI ** (1 - m)
    # real-space part (formula 47, kamstr.f:281-305)
    for rv in lat.rvecs(rcut, centre=(-sx, -sy)):
        rx, ry = rv
        ex1 = np.exp(-CI * (rx * kx + ry * ky))
        rsv = (rx + sx, ry + sy, sz)
        rs = math.sqrt(rsv[0] ** 2 + rsv[1] ** 2 + rsv[2] ** 2)
        if rs < 1e-5:
            continue
        ylm = ylmc(rsv, lmax2)
        intil = ilkam(lmax2, alpha, rs, kappa)
        a = -kappa * rs / 2.0
        b = ex1 * cs2 / a
        for l in range(lmax2 + 1):
            b = b * a
            c = intil[l] * b
            sl = slice(l * l, (l + 1) ** 2)
            dlm2[sl] += c * np.conj(ylm[sl])
    return dlm1 + dlm2


def kamstr(e: complex, kx: float, ky: float, lmax: int, sep, lat: Lattice2D, factor: float = 1.0,
           gcut: float = 12.0, rcut: float = 40.0) -> np.ndarray:
    """main/kamstr.f:20-392: alm[lm1, lm2] = sum_L gau[lm1, lm2, L] D_L(k, sep)."""
    d = kambe_dlm(e, kx, ky, sep, 2 * lmax, lat, factor, gcut, rcut)
    return np.tensordot(gauntcalc(lmax), d, axes=([2], [0]))


_GAUNT_OURS: dict = {}


def _gaunt_ours(lmax: int) -> np.ndarray:
    """C[L, L', L''] = <Y_L Y*_L' Y_L''> (complex Y_lm of ylmc) by quadrature."""
    if lmax in _GAUNT_OURS:
        return _GAUNT_OURS[lmax]
    l2 = 2 * lmax
    nq = (4 * lmax + l2) // 2 + 2
    xg, wg = np.polynomial.legendre.leggauss(nq)
    nph = 4 * lmax + l2 + 2
    out = np.zeros(((lmax + 1) ** 2, (lmax + 1) ** 2, (l2 + 1) ** 2), complex)
    for ct, wq in zip(xg, wg):
        st = math.sqrt(1 - ct * ct)
        for p in range(nph):
            phi = 2 * math.pi * p / nph
            v = (st * math.cos(phi), st * math.sin(phi), ct)
            y2 = ylmc(v, l2)
            y1 = y2[:(lmax + 1) ** 2]
            out += (wq * 2 * math.pi / nph) * y1[:, None, None] * np.conj(y1)[None, :, None] * y2[None, None, :]
    out[np.abs(out) < 1e-13] = 0.0
    _GAUNT_OURS[lmax] = out
    return out


def alm_coef(lmax: int) -> np.ndarray:
    """coef[L, L', q] with alm(k, s) = sum_q coef[L, L', q] D_q(k, s): the
    mapping of lattice_g folded into one tensor (4 pi <Y_L Y*_L' Y_L''>
    i^(l'-l-l'') (-1)^(l''+m'') at q = (l'', -m''))."""
    l2 = 2 * lmax
    lv = np.array([l for l in range(lmax + 1) for _ in range(-l, l + 1)])
    lv2 = np.array([l for l in range(l2 + 1) for _ in range(-l, l + 1)])
    mv2 = np.array([m for l in range(l2 + 1) for m in range(-l, l + 1)])
    neg = np.array([l * (l + 1) - m for l in range(l2 + 1) for m in range(-l, l + 1)])
    ph = (1j) ** ((-lv[:, None, None] + lv[None, :, None] - lv2[None, None, :]) % 4)
    t = 4 * math.pi * _gaunt_ours(lmax) * ph * ((-1.0) ** (mv2 + lv2))[None, None, :]
    out = np.zeros_like(t)
    out[:, :, neg] = t
    return out


def lattice_g(e: complex, kx: float, ky: float, lmax: int, sep, lat: Lattice2D, **cut) -> np.ndarray:
    """sum_R e^{ik.R} G0_{LL'}(R + sep) with the free-space constants
    G0_{LL'}(r) = -4 pi i kappa sum_L'' <Y_L Y*_L' Y_L''> i^(l'-l-l'') h_l''(kappa r) Y_L''(r)
    (the convention of the screened tables the GPU path transforms), from the
    Kambe sums: kambe_dlm(-k, sep) = -i kappa (-1)^l sum_R e^{ik.R} h_l Y*_L(R + sep)
    and Y_lm = (-1)^m Y*_l,-m.  The reference's own alm(k, sep) of kamstr.f is the
    same sum at -k."""
    l2 = 2 * lmax
    lv = np.array([l for l in range(lmax + 1) for _ in range(-l, l + 1)])
    lv2 = np.array([l for l in range(l2 + 1) for _ in range(-l, l + 1)])
    mv2 = np.array([m for l in range(l2 + 1) for m in range(-l, l + 1)])
    neg = np.array([l * (l + 1) - m for l in range(l2 + 1) for m in range(-l, l + 1)])
    d = kambe_dlm(e, -kx, -ky, sep, l2, lat, **cut)
    ph = (1j) ** ((-lv[:, None, None] + lv[None, :, None] - lv2[None, None, :]) % 4)
    p = (-1.0) ** (mv2 + lv2) * d[neg]
    return 4 * math.pi * np.tensordot(_gaunt_ours(lmax) * ph, p, axes=([2], [0]))


def gstore_block(e: complex, kx: float, ky: float, lmax: int, sep, lat: Lattice2D) -> np.ndarray:
    """alm(k, sep) the way main/gstore.f:146-170 evaluates block (a, b) of
    gtotal for sep = c_a - c_b: the plane-wave sum of directg.f when
    |s_z| |b|_min >= 5 (its gp for s_z > 0, its gm of -sep otherwise), else
    the Kambe sums of kamstr.f."""
    s = np.asarray(sep, float)
    if abs(s[2]) * lat.bmin >= 5.0:
        if s[2] > 0:
            return directg(e, kx, ky, lmax, s, lat)[0]
        return directg(e, kx, ky, lmax, -s, lat)[1]
    return kamstr(e, kx, ky, lmax, s, lat)


def screened_slab(e: complex, kx: float, ky: float, lmax: int, pos, alpha, lat: Lattice2D) -> np.ndarray:
    """main/gstore.f:146-185 + main/scrstr.f:2-138: the layer-pair constants of
    a slab of layers at positions pos (nl, 3), screened as
    G' = G (1 - alpha G)^-1 with alpha[a, l] per layer and l.

    Block (a, b) is gstore's alm(k, pos_a - pos_b) times the in-plane phase
    e^{ik.(pos_b - pos_a)}: the Bloch sum over the sites R_b = pos_b + R of
    layer b of G0(pos_a - R_b) with the phase e^{ik.(R_b - pos_a)} of the full
    site vectors, the orientation (G_nm = G0(R_n - R_m)) and phase convention
    of the real-space screened tables.  Returns (nl, nl, lmmax, lmmax)."""
    pos = np.asarray(pos, float)
    nl, lm = len(pos), (lmax + 1) ** 2
    lv = np.array([l for l in range(lmax + 1) for _ in range(-l, l + 1)])
    cache = {}
    g = np.zeros((nl * lm, nl * lm), complex)
    for a in range(nl):
        for b in range(nl):
            s = tuple(np.round(pos[a] - pos[b], 10))
            if s not in cache:
                cache[s] = gstore_block(e, kx, ky, lmax, s, lat)
            ph = np.exp(1j * (kx * (pos[b][0] - pos[a][0]) + ky * (pos[b][1] - pos[a][1])))
            g[a * lm:(a + 1) * lm, b * lm:(b + 1) * lm] = ph * cache[s]
    al = np.concatenate([np.asarray(alpha[a], complex)[lv] for a in range(nl)])
    gs = g @ np.linalg.inv(np.eye(nl * lm) - al[:, None] * g)
    return gs.reshape(nl, lm, nl, lm).transpose(0, 2, 1, 3)


def sphrm(ct: complex, st: complex, cf: complex, lmax: int) -> np.ndarray:
    """main/sphrm.f: Y_lm for the complex angles (cos, sin, e^{i phi}) of an
    evanescent wave vector, by the explicit m = l, l-1 forms and the
    recurrence in l; index l(l+1)+m."""
    y = np.zeros((lmax + 1) ** 2 + 1, complex)      # 1-based as in the Fortran
    y[1] = math.sqrt(0.25 / math.pi)
    if lmax == 0:
        return y[1:]
    a = b = asg = 1.0
    sf = sa = 1.0 + 0j
    lp = 1
    for l in range(1, lmax + 1):
        fl = float(l)
        a = 0.5 * a * fl * (2.0 * fl - 1.0)
        b = fl * b
        asg = -asg
        lm = lp + 1
        lp = lp + l + l + 1
        sf = sf * cf
        fac = math.sqrt((2.0 * fl + 1.0) * a / (4.0 * math.pi * b * b)) * sa
        y[lm] = fac * st / sf
        y[lp] = asg * fac * st * sf
        fac = math.sqrt(2.0 * fl) * fac * ct
        y[lm + 1] = fac * cf / sf
        y[lp - 1] = -asg * fac * sf / cf
        sa = sa * st
    if lmax == 1:
        return y[1:]
    for m in range(2, lmax + 1):
        mm = m + m - 4
        fm = float(m - 2)
        a = math.sqrt(1.0 / (fm + fm + 3.0))
        ln = m * m - 1
        lm = ln - m - m + 2
        for l in range(m, lmax + 1):
            fl = float(l)
            b = math.sqrt((fl + fm) * (fl - fm) / ((fl + fl + 1.0) * (fl + fl - 1.0)))
            lp = ln + l + l
            y[lp] = (ct * y[ln] - a * y[lm]) / b
            y[lp - mm] = (ct * y[ln - mm] - a * y[lm - mm]) / b
            a = b
            lm = ln
            ln = lp
    return y[1:]


def directg(e: complex, kx: float, ky: float, lmax: int, sep, lat: Lattice2D, gcut: float = 30.0):
    """main/directg.f:2-151: the plane-wave form of the layer-pair sums that
    gstore.f:158-166 uses when |s_z| |b|_min >= 5 (s_z > 0).  Returns
    (gp, gm): gp is block (j, i) and gm block (i, j) of gtotal for
    sep = c_j - c_i, i.e. alm(k, sep) and alm(k, -sep) of kamstr."""
    lmx2 = (lmax + 1) ** 2
    kappa2 = complex(e)
    kappa = np.sqrt(kappa2)
    f1 = 8.0 * math.pi * math.pi / lat.area
    gp = np.zeros((lmx2, lmx2), complex)
    gm = np.zeros((lmx2, lmx2), complex)
    s1, s2, s3 = (float(t) for t in sep)
    lv = np.array([l for l in range(lmax + 1) for _ in range(-l, l + 1)])
    mv = np.array([m for l in range(lmax + 1) for m in range(-l, l + 1)])
    neg = np.array([l * (l + 1) - m for l in range(lmax + 1) for m in range(-l, l + 1)])
    sl, il, sm = (-1.0) ** lv, (1j) ** lv, (-1.0) ** mv
    for g in lat.gvecs(gcut, centre=(-kx, -ky)):
        gkx, gky = g[0] + kx, g[1] + ky
        gk2 = gkx * gkx + gky * gky
        gk = math.sqrt(gk2)
        gkz = np.sqrt(kappa2 - gk2)
        phi = (gkx + 1j * gky) / gk if gk > 1e-6 else 1.0 + 0j
        y = sphrm(gkz / kappa, gk / kappa, phi, lmax)
        ylm1 = sl * il * y
        ylm2 = il * sm * y[neg]
        ylm3 = il * sm * y
        ylm4 = sl * il * y[neg]
        fp = np.exp(1j * (gkx * s1 + gky * s2 + gkz * s3)) * f1 / gkz
        fm = np.exp(1j * (-gkx * s1 - gky * s2 + gkz * s3)) * f1 / gkz
        # gp(lmj, lmi) += ylm1(lmi) fp ylm2(lmj) (-i)
        gp += -1j * fp * np.outer(ylm2, ylm1)
        gm += -1j * fm * np.outer(ylm4, ylm3)
    return gp, gm


def slab_table_blocks(e: complex, kx: float, ky: float, lmax: int, pos, alpha, lat: Lattice2D, blk_of_j: dict,
                      centre: int) -> np.ndarray:
    """The reference's G_scr(k) in the block layout of the real-space tables:
    block blk_of_j[j] = screened slab block (centre, centre + j), the layer
    offsets -jmax..jmax that gstore.f:236-282 keeps of gtotal as g2d."""
    gs = screened_slab(e, kx, ky, lmax, pos, alpha, lat)
    lm = (lmax + 1) ** 2
    out = np.zeros((len(blk_of_j), lm, lm), complex)
    for j, b in blk_of_j.items():
        out[b] = gs[centre, centre + j]
    return out
