"""Generates tests/golden/analytic_cases.json: one SPH step of small hand-placed particle
sets, evaluated in 50-digit arithmetic (mpmath) from the reference's formulas.

This is an independent restatement (Python, real arithmetic) of the step that the
reference's CPU simulator performs (src/CCPUParticleSimulator.cpp:9-229, walls from
src/CCollisionGeometry.cpp:117-133, constants include/CParticle.h:80-84, dt
src/CBaseParticleSimulator.cpp:7). The reference itself cannot run here (Qt5/Qt3D
absent), so these vectors pin the C oracle's formulas, not the reference's binaries.

Inputs are float32 values; the constants are the float32 values the reference uses;
the neighbour set is the reference's: particles in the 27 cells around a particle's
clamped cell (cell size h, cell = floor((p + box/2) / h) in double), r^2 <= h^2.

    python tests/golden/make_analytic.py
"""
import json
import math
import os

import mpmath as mp
import numpy as np

mp.mp.dps = 50
HERE = os.path.dirname(os.path.abspath(__file__))

f32 = np.float32
H = f32(0.0457)
MASS = f32(0.02)
K = f32(3.0)
RHO0 = f32(998.29)
MU = f32(3.5)
DT = f32(0.01)
WALL_K = 10000.0
WALL_DAMPING = -0.9
WALL_R = 0.01


def M(x):
    return mp.mpf(float(x))


def grid_res(box):
    return [int(math.ceil(f32(b) / H)) for b in box]  # float division, ceil


def cell_axis(p, box, res):
    q = (float(f32(p)) + float(f32(box)) / 2.0) / float(H)
    if not q >= 0.0:
        return 0
    if q >= res:
        return res - 1
    return int(math.floor(q))


def step(box, gravity, pos, vel):
    n = len(pos)
    res = grid_res(box)
    cells = [[cell_axis(pos[i][a], box[a], res[a]) for a in range(3)] for i in range(n)]
    h, h2 = M(H), M(H) * M(H)
    cp = mp.mpf(315) / (64 * mp.pi * h ** 9)
    cs = mp.mpf(-45) / (mp.pi * h ** 6)
    cv = mp.mpf(45) / (mp.pi * h ** 6)
    P = [[M(c) for c in p] for p in pos]
    V = [[M(c) for c in v] for v in vel]

    def adjacent(i, j):
        return all(abs(cells[i][a] - cells[j][a]) <= 1 for a in range(3))

    def diff(a, b):
        return [a[k] - b[k] for k in range(3)]

    rho, prs = [], []
    for i in range(n):
        s = mp.mpf(0)
        for j in range(n):
            if not adjacent(i, j):
                continue
            d = diff(P[i], P[j])
            r2 = sum(x * x for x in d)
            if r2 <= h2:
                s += cp * (h2 - r2) ** 3
        r = M(MASS) * s
        rho.append(r)
        prs.append(M(K) * (r - M(RHO0)))
    acc, scale = [], []
    g = [M(x) for x in gravity]
    half = [M(f32(b)) / 2 for b in box]
    for i in range(n):
        fp = [mp.mpf(0)] * 3
        fv = [mp.mpf(0)] * 3
        mp_abs = mp.mpf(0)
        mv_abs = mp.mpf(0)
        for j in range(n):
            if j == i or not adjacent(i, j):
                continue
            d = diff(P[i], P[j])
            r2 = sum(x * x for x in d)
            if r2 <= h2:
                r = mp.sqrt(r2)
                pij = prs[i] / rho[i] ** 2 + prs[j] / rho[j] ** 2
                tp = [pij * cs * (h - r) ** 2 * x / r for x in d]
                tv = [(V[j][k] - V[i][k]) * cv * (h - r) / rho[j] for k in range(3)]
                fp = [fp[k] + tp[k] for k in range(3)]
                fv = [fv[k] + tv[k] for k in range(3)]
                mp_abs += mp.sqrt(sum(x * x for x in tp))
                mv_abs += mp.sqrt(sum(x * x for x in tv))
        a = [(-M(MASS) * rho[i] * fp[k] + M(MU) * M(MASS) * fv[k] + g[k] * rho[i]) / rho[i] for k in range(3)]
        wall_abs = mp.mpf(0)
        for w in range(6):
            ax = w % 3
            inv = 1 if w < 3 else -1
            wp = -half[ax] if w < 3 else half[ax]
            d = (wp - P[i][ax]) * inv + mp.mpf(WALL_R)
            if d > 0:
                t1 = mp.mpf(WALL_K) * inv * d
                t2 = mp.mpf(WALL_DAMPING) * (V[i][ax] * inv) * inv
                a[ax] += t1 + t2
                wall_abs += abs(t1) + abs(t2)
        acc.append(a)
        sc = (mp_abs * M(MASS) * abs(rho[i]) + mv_abs * M(MU) * M(MASS)) / abs(rho[i])
        scale.append(sc + mp.sqrt(sum(x * x for x in g)) + wall_abs)
    dt = M(DT)
    pos_new = [[P[i][k] + V[i][k] * dt + acc[i][k] * dt * dt for k in range(3)] for i in range(n)]
    vel_new = [[(pos_new[i][k] - P[i][k]) / dt for k in range(3)] for i in range(n)]
    fmt = lambda x: float(x)
    return {
        "cells": cells, "res": res,
        "rho": [fmt(x) for x in rho], "p": [fmt(x) for x in prs],
        "acc": [[fmt(x) for x in a] for a in acc], "acc_scale": [fmt(x) for x in scale],
        "pos_new": [[fmt(x) for x in p] for p in pos_new], "vel_new": [[fmt(x) for x in v] for v in vel_new],
    }


def as_f32(rows):
    return [[float(f32(x)) for x in r] for r in rows]


def cases():
    g0 = [0.0, float(f32(-9.80665)), 0.0]
    out = []
    out.append(("single", [1.0, 1.0, 1.0], g0, [[0.0, 0.0, 0.0]], [[0.0, 0.0, 0.0]]))
    out.append(("pair_x", [1.0, 1.0, 1.0], g0, [[-0.01, 0.0, 0.0], [0.012, 0.0, 0.0]],
                [[0.1, 0.0, 0.0], [-0.2, 0.05, 0.0]]))
    out.append(("triangle", [1.0, 1.0, 1.0], g0, [[0.0, 0.0, 0.0], [0.02, 0.005, -0.003], [0.004, 0.021, 0.011]],
                [[0.0, 0.1, 0.0], [0.3, -0.2, 0.1], [-0.1, 0.0, 0.25]]))
    out.append(("near_wall", [0.4, 0.4, 0.4], g0, [[-0.195, 0.0, 0.0], [-0.17, 0.004, -0.002]],
                [[-0.3, 0.0, 0.1], [0.0, 0.0, 0.0]]))
    out.append(("corner_outside", [0.4, 0.4, 0.4], g0,
                [[-0.2005, -0.2003, -0.2001], [-0.18, -0.19, -0.195], [-0.205, -0.185, -0.19]],
                [[-0.1, -0.2, 0.0], [0.0, 0.0, 0.0], [0.05, 0.0, -0.05]]))
    # particles straddling the x = 0 cell face of a 0.4 m box: (p + 0.2) / h is ~4.376
    out.append(("non_cubic_box", [0.5, 0.3, 0.2], [0.0, -9.81, 0.0],
                [[0.0, 0.0, 0.0], [0.03, 0.01, 0.0], [-0.02, 0.015, 0.01], [0.01, -0.02, -0.015]],
                [[0.0, 0.0, 0.0], [0.1, 0.0, 0.0], [0.0, -0.1, 0.0], [0.0, 0.0, 0.2]]))
    rng = np.random.default_rng(20171)
    pos = (rng.uniform(-1.5, 1.5, size=(20, 3)) * float(H)).astype(np.float32)
    vel = rng.normal(0, 0.3, size=(20, 3)).astype(np.float32)
    out.append(("cluster20", [1.0, 1.0, 1.0], [0.0, -9.81, 0.0], pos.tolist(), vel.tolist()))
    return out


def main():
    res = []
    for name, box, g, pos, vel in cases():
        box32 = [float(f32(b)) for b in box]
        g32 = [float(f32(x)) for x in g]
        pos32, vel32 = as_f32(pos), as_f32(vel)
        r = step(box32, g32, pos32, vel32)
        r.update({"name": name, "box": box32, "gravity": g32, "pos": pos32, "vel": vel32})
        res.append(r)
    path = os.path.join(HERE, "analytic_cases.json")
    with open(path, "w") as f:
        json.dump({"generator": "tests/golden/make_analytic.py", "digits": 50, "cases": res}, f, indent=1)
    print(path, len(res), "cases")


if __name__ == "__main__":
    main()
