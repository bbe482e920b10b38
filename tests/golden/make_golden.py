"""Generates tests/golden/analytic.json: known answers for the oracle.

GPUCell ships no golden vectors (no tests, no run outputs), so the oracle is
pinned to quantities that follow from the published formulas alone,
computed here independently of oracle/oracle.c:

* Wendland C2 values W(r) and F(r) = -W'(r)/r at a few radii (exact
  rational arithmetic times 1/pi);
* the regular icosahedron (the level-0 icosphere): area, volume and
  dihedral angle;
* the WLC-POW spring constants of one edge (zero force at l0, the linear
  shear-modulus relation of Fedosov et al. 2010);
* the SDPD force between two fluid particles (Espanol & Revenga 2003) with
  the noise off, written out term by term;
* Philox4x32-10 and Philox2x32-10 outputs and the per-step noise key
  (SplitMix64 finaliser) from from-scratch Python implementations of the
  published round functions (Salmon et al. 2011; Steele, Lea & Flood 2014).

Run:  python tests/golden/make_golden.py
"""
import json
import math
import os
from fractions import Fraction as Fr

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "analytic.json")


def wendland(r, rc=1.0):
    s = Fr(r) / Fr(rc)
    t = 1 - s
    W = Fr(21, 2) * t ** 4 * (1 + 4 * s) / Fr(rc) ** 3      # times 1/pi
    F = Fr(210) * t ** 3 / Fr(rc) ** 5                       # times 1/pi
    return float(W) / math.pi, float(F) / math.pi


def icosahedron():
    a = 4.0 / math.sqrt(10.0 + 2.0 * math.sqrt(5.0))         # edge for circumradius 1
    return dict(edge=a, area=5.0 * math.sqrt(3.0) * a * a, volume=5.0 / 12.0 * (3.0 + math.sqrt(5.0)) * a ** 3,
                dihedral=math.acos(-math.sqrt(5.0) / 3.0))


def wlc_pow(l0, mu0, kT, x0=1 / 2.2, m=2.0):
    u = 1.0 - x0
    kw = 1.0 / (4 * u * u) - 0.25 + x0
    km = x0 / (2 * u ** 3) - 1.0 / (4 * u * u) + 0.25
    C = math.sqrt(3.0) / (4.0 * l0) * (km + (m + 1.0) * kw)
    p = kT * C / mu0
    kp = (kT / p) * l0 ** m * kw
    return dict(l0=l0, mu0=mu0, kT=kT, lmax=l0 / x0, p=p, kp=kp)


def sdpd_pair(xi, xj, vi, vj, rho_i, rho_j, P_i, P_j, eta, zeta, m=1.0, rc=1.0):
    d = [a - b for a, b in zip(xi, xj)]
    r = math.sqrt(sum(x * x for x in d))
    e = [x / r for x in d]
    s = r / rc
    F = 210.0 / (math.pi * rc ** 5) * (1 - s) ** 3
    di, dj = rho_i / m, rho_j / m
    A = 5.0 * eta / 3.0 - zeta
    B = 5.0 * (zeta + eta / 3.0)
    vij = [a - b for a, b in zip(vi, vj)]
    ev = sum(a * b for a, b in zip(e, vij))
    cons = (P_i / di ** 2 + P_j / dj ** 2) * F
    fdd = F / (di * dj)
    return [cons * d[k] - fdd * (A * vij[k] + B * ev * e[k]) for k in range(3)]


M32 = 0xFFFFFFFF


def philox(ctr, key, rounds=10):
    c = list(ctr)
    k = list(key)
    for _ in range(rounds):
        p0 = 0xD2511F53 * c[0]
        p1 = 0xCD9E8D57 * c[2]
        c = [((p1 >> 32) ^ c[1] ^ k[0]) & M32, p1 & M32, ((p0 >> 32) ^ c[3] ^ k[1]) & M32, p0 & M32]
        k = [(k[0] + 0x9E3779B9) & M32, (k[1] + 0xBB67AE85) & M32]
    return c


def philox2(ctr, key, rounds=10):
    c0, c1, k = ctr[0], ctr[1], key
    for _ in range(rounds):
        pr = 0xD256D193 * c0
        c0, c1 = ((pr >> 32) ^ k ^ c1) & M32, pr & M32
        k = (k + 0x9E3779B9) & M32
    return [c0, c1]


M64 = (1 << 64) - 1


def splitmix_mix(z):
    z = (z + 0x9E3779B97F4A7C15) & M64
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
    return z ^ (z >> 31)


def noise_key(seed, step):
    return splitmix_mix((seed * 0x9E3779B97F4A7C15 + step) & M64) >> 32


def main():
    radii = [0.0, 0.125, 0.25, 0.5, 0.75, 0.9]
    g = dict(
        wendland=[dict(r=r, W=wendland(r)[0], F=wendland(r)[1]) for r in radii],
        icosahedron=icosahedron(),
        wlc_pow=[wlc_pow(0.35, 100.0, 1.0), wlc_pow(0.12, 6.3, 0.5)],
        sdpd_pair=[],
        philox=[],
    )
    cases = [((0.1, 0.2, 0.3), (0.5, -0.1, 0.25), (1.0, 0.0, -0.5), (-0.5, 0.25, 0.0), 27.3, 26.8, 4.0, -3.5, 10.0, 0.0),
             ((2.0, 2.0, 2.0), (2.3, 1.8, 2.4), (0.0, 0.1, 0.0), (0.2, 0.0, 0.0), 27.0, 27.0, 0.0, 0.0, 5.0, 1.0)]
    for xi, xj, vi, vj, ri, rj, pi, pj, eta, zeta in cases:
        g["sdpd_pair"].append(dict(xi=xi, xj=xj, vi=vi, vj=vj, rho_i=ri, rho_j=rj, P_i=pi, P_j=pj, eta=eta, zeta=zeta,
                                   force_i=sdpd_pair(xi, xj, vi, vj, ri, rj, pi, pj, eta, zeta)))
    for ctr, key in (([0, 0, 0, 0], [0, 0]), ([1, 2, 3, 4], [5, 6]), ([7, 123456, 42, 0], [1, 0]),
                     ([M32, M32, M32, M32], [M32, M32])):
        g["philox"].append(dict(ctr=ctr, key=key, out=philox(ctr, key)))
    g["philox2"] = [dict(ctr=c, key=k, out=philox2(c, k)) for c, k in
                     (([0, 0], 0), ([1, 2], 3), ([123456, 7654321], 0xDEADBEEF), ([M32, M32], M32))]
    g["noise_key"] = [dict(seed=sd, step=st, key=noise_key(sd, st)) for sd, st in ((1, 0), (1, 1), (1, 17),
                                                                                  (12345, 999), (2 ** 40 + 3, 5))]
    with open(OUT, "w") as f:
        json.dump(g, f, indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
