"""Generates tests/golden/golden.json: golden vectors for the oracle.

An independent pure-Python restatement of maikel/FiniteVolumeSolver's
perfect-gas MUSCL-Hancock / HLLE / Einfeldt / update arithmetic (Python
floats are IEEE doubles with correctly rounded + - * / sqrt and no FMA, like
the reference's SSE2 build).  Small cases only; values are stored as hex
floats so comparisons are bit-exact.

Reference formulas:
  src/equations/PerfectGas.cpp:25-124          CompleteFromCons, Flux
  src/equations/perfect_gas/EinfeldtSignalVelocities.hpp:64-97
  include/fub/flux_method/HllMethod.hpp:260-293, 337-347
  include/fub/flux_method/MusclHancockMethod.hpp:92-187, 419-485
  include/fub/flux_method/FluxMethod.hpp:200-215, 295-314
  src/HyperbolicPatchIntegrator.cpp:88-105
Reference tests whose setups are reproduced:
  tests/test.HyperbolicSplitPatchIntegrator.cpp:37-71 (update hand vectors)
  tests/test.simd_FluxMethod.cpp:54-105 (single MUSCL stencil, MinMod)
  tests/test.simd_FluxMethod.cpp:107-186 (HLLE on a 16x16 sin-energy patch)

Run:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import math
import random
from pathlib import Path

GAMMA = 1.4
GM1INV = 1.0 / (1.4 - 1.0)


def sqn(m):
    if len(m) == 1:
        return m[0] * m[0]
    if len(m) == 2:
        return m[0] * m[0] + m[1] * m[1]
    return m[0] * m[0] + (m[1] * m[1] + m[2] * m[2])


def complete(u):
    D = len(u) - 2
    rho, m, E = u[0], list(u[1:1 + D]), u[1 + D]
    e_kin = 0.5 * sqn(m) / rho
    p = (E - e_kin) / GM1INV
    c = math.sqrt(GAMMA * p / rho)
    return [rho, *m, E, p, c]


def flux(q, d):
    D = len(q) - 4
    rho, m, E, p = q[0], q[1:1 + D], q[1 + D], q[2 + D]
    v = m[d] / rho
    f = [m[d]] + [v * m[k] for k in range(D)] + [v * (E + p)]
    f[1 + d] += p
    return f


def pmin(a, b):
    return a if a < b else b


def pmax(a, b):
    return a if a > b else b


def einfeldt(L, R, d):
    D = len(L) - 4
    rhoL, rhoR = L[0], R[0]
    sqL, sqR = math.sqrt(rhoL), math.sqrt(rhoR)
    oo = 1.0 / (sqL + sqR)
    uL, uR = L[1 + d] / rhoL, R[1 + d] / rhoR
    roeU = (uL * sqL + uR * sqR) * oo
    hL = (L[1 + D] + L[2 + D]) / rhoL
    hR = (R[1 + D] + R[2 + D]) / rhoR
    roeH = (hL * sqL + hR * sqR) * oo
    roeA = math.sqrt((GAMMA - 1.0) * (roeH - 0.5 * roeU * roeU))
    return pmin(uL - L[3 + D], roeU - roeA), pmax(roeU + roeA, uR + R[3 + D])


def hll(L, R, d):
    D = len(L) - 4
    s0, s1 = einfeldt(L, R, d)
    fL, fR = flux(L, d), flux(R, d)
    sL, sR = pmin(s0, 0.0), pmax(s1, 0.0)
    sLsR = sL * sR
    ds = sR - sL
    ds = ds if ds > 0.0 else 1.0
    return [(sR * fL[k] - sL * fR[k] + sLsR * (R[k] - L[k])) / ds for k in range(D + 2)]


def hll_dt(L, R, dx, d):
    s0, s1 = einfeldt(L, R, d)
    return dx / pmax(pmax(0.0, abs(s0)), abs(s1))


def slope(lim, a, b, c):
    sL, sR = b - a, c - b
    if lim == "van_leer":
        r = 2.0 * sL * sR
        return r / (sL + sR) if r > 0.0 else 0.0
    return pmax(0.0, pmin(sL, sR)) if sR > 0 else pmin(0.0, pmax(sL, sR))


def predict(q0, q1, q2, lim, lh, d, side):
    K = len(q1)
    s = [slope(lim, q0[k], q1[k], q2[k]) for k in range(K)]
    uL = [q1[k] - 0.5 * s[k] for k in range(K)]
    uR = [q1[k] + 0.5 * s[k] for k in range(K)]
    fL, fR = flux(complete(uL), d), flux(complete(uR), d)
    base = uR if side > 0 else uL
    return complete([base[k] + lh * (fL[k] - fR[k]) for k in range(K)])


def muscl(st, dt, dx, d, lim):
    """st: 4 conservative states along d."""
    lh = 0.5 * dt / dx
    r0 = predict(st[0], st[1], st[2], lim, lh, d, +1)
    r1 = predict(st[1], st[2], st[3], lim, lh, d, -1)
    return hll(r0, r1, d)


def hexs(v):
    return [float(x).hex() for x in v]


def sin_patch_states(nx, ny, dx, grow_dir):
    """tests/test.simd_FluxMethod.cpp:107-131: cells [0,16)^2 grown by 1 in
    grow_dir; rho = 1, m = 0, E = 1 + 0.5 sin(x^2 + y^2) with x = i dx."""
    lo = [0, 0]
    hi = [nx, ny]
    lo[grow_dir] -= 1
    hi[grow_dir] += 1
    cells = {}
    for j in range(lo[1], hi[1]):
        for i in range(lo[0], hi[0]):
            x, y = float(i) * dx, float(j) * dx
            E = 1.0 + 0.5 * math.sin(x * x + y * y)
            cells[(i, j)] = complete([1.0, 0.0, 0.0, E])
    return lo, hi, cells


def main():
    out = {}
    # update hand vectors (test.HyperbolicSplitPatchIntegrator.cpp:37-71)
    out["update_1cell"] = {"prev": [1.0], "flux": [0.3, 0.4], "next": hexs([1.0 + 1.0 * (0.3 - 0.4)])}
    prev8 = [1.0] * 8
    f9 = [0.3, 0.4, -0.2, 0.0, 0.1, 0.2, 0.0, 0.0, 0.0]
    out["update_8cell"] = {"prev": prev8, "flux": f9,
                           "next": hexs([prev8[i] + 1.0 * (f9[i] - f9[i + 1]) for i in range(8)])}

    # single MUSCL stencil, MinMod (test.simd_FluxMethod.cpp:54-105)
    a = [1.0, 0.0, 0.0, 2.0]
    b = [1.0, 0.0, 0.0, 1.0]
    out["muscl_minmod_single"] = {"stencil": [a, a, b, b], "dt": 1.0, "dx": 1.0,
                                  "flux": hexs(muscl([a, a, b, b], 1.0, 1.0, 0, "minmod"))}

    # HLLE patch fluxes, 16x16 sin-energy patch, X and Y; dt from the
    # sequential HllMethod::ComputeStableDt (test.simd_FluxMethod.cpp:107-186)
    dx = 0.0125
    for d, name in ((0, "X"), (1, "Y")):
        lo, hi, cells = sin_patch_states(16, 16, dx, d)
        # sequential dt: windows of 2 cells starting in Shrink(box, d, {0, 2})
        dt = math.inf
        for j in range(lo[1], hi[1] - (2 if d == 1 else 0)):
            for i in range(lo[0], hi[0] - (2 if d == 0 else 0)):
                c0 = (i, j)
                c1 = (i + 1, j) if d == 0 else (i, j + 1)
                dt = min(hll_dt(cells[c0], cells[c1], dx, d), dt)
        fl = [0, 0]
        fh = [16, 16]
        fh[d] += 1
        fluxes = []
        for j in range(fl[1], fh[1]):
            for i in range(fl[0], fh[0]):
                L = (i - 1, j) if d == 0 else (i, j - 1)
                fluxes.append(hll(cells[L], cells[(i, j)], d))
        # component-major
        comp = [[f[k] for f in fluxes] for k in range(4)]
        out[f"hlle_sin16_{name}"] = {"dt": dt.hex(), "dx": dx, "cell_lo": lo, "cell_hi": hi,
                                     "face_lo": fl, "face_hi": fh,
                                     "fluxes": [hexs(c) for c in comp]}

    # 3-D MUSCL-VanLeer-HLLE fluxes of random stencils (checks the 3-term
    # kinetic-energy summation order)
    rng = random.Random(12345)
    sten = []
    res = []
    for _ in range(16):
        st = []
        for _s in range(4):
            rho = rng.uniform(0.1, 2.0)
            v = [rng.uniform(-0.5, 0.5) for _ in range(3)]
            p = rng.uniform(0.1, 2.0)
            E = p * GM1INV + 0.5 * rho * sqn(v)
            st.append([rho, rho * v[0], rho * v[1], rho * v[2], E])
        for d in range(3):
            res.append(hexs(muscl(st, 0.01, 0.05, d, "van_leer")))
        sten.append(st)
    out["muscl_vanleer_3d_random"] = {"dt": 0.01, "dx": 0.05, "stencils": sten, "fluxes": res}

    path = Path(__file__).with_name("golden.json")
    path.write_text(json.dumps(out, indent=1))
    print(f"wrote {path}")


if __name__ == "__main__":
    main()
