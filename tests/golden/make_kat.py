"""Generates tests/golden/kat_*.json: known-answer cases for the PBF formulas.

Independent FP64 restatement of the reference kernels' formulas, written from
the reference source (sim/pbf_lambda.cu:38-107, sim/pbf_delta_apply.cu:40-112,
sim/xsph.cu:39-95, sim/boundary.cu:11-25, sim/hash_keys.cu:14-27) without
using the oracle library, so that the oracle is checked against it.  Each case
is a handful of particles whose answer can be followed by hand.

Run:  python tests/golden/make_kat.py
"""
import json
import math
import os
import struct

HERE = os.path.dirname(os.path.abspath(__file__))


def kernel(h):
    return {
        "h": h,
        "h2": h * h,
        "poly6": 315.0 / (64.0 * math.pi * h ** 9),
        "spiky": 15.0 / (math.pi * h ** 6),
    }


def cell_of(p, mins, cs, dim):
    c = [int(math.floor((p[a] - mins[a]) / cs)) for a in range(3)]
    return [max(0, min(c[a], dim[a] - 1)) for a in range(3)]


def key_of(c, dim):
    return (c[2] * dim[1] + c[1]) * dim[0] + c[0]


def neighbour_order(pos, mins, cs, dim):
    """Reference candidate order for each particle: dz,dy,dx then stable
    sorted order of (key, id)."""
    keys = [key_of(cell_of(p, mins, cs, dim), dim) for p in pos]
    order = sorted(range(len(pos)), key=lambda i: (keys[i], i))
    out = {}
    for i in range(len(pos)):
        ci = cell_of(pos[i], mins, cs, dim)
        cand = []
        for dz in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dx in (-1, 0, 1):
                    c = [ci[0] + dx, ci[1] + dy, ci[2] + dz]
                    if any(c[a] < 0 or c[a] >= dim[a] for a in range(3)):
                        continue
                    k = key_of(c, dim)
                    cand += [j for j in order if keys[j] == k]
        out[i] = cand
    return out, keys, order


def lam_of(i, pos, order, kc, m, rho0, eps, cap, lam_max):
    dens, g, sg2, contrib = 0.0, [0.0, 0.0, 0.0], 0.0, 0
    for j in order[i]:
        if cap > 0 and contrib >= cap:
            break
        if j == i:
            continue
        r = [pos[i][a] - pos[j][a] for a in range(3)]
        r2 = sum(x * x for x in r)
        if r2 > kc["h2"]:
            continue
        contrib += 1
        dens += m * kc["poly6"] * (kc["h2"] - r2) ** 3
        rr = math.sqrt(r2)
        coeff = -3.0 * kc["spiky"] * (kc["h"] - rr) ** 2 / max(rr, 1e-6)
        gr = [coeff * x for x in r]
        g = [g[a] + gr[a] for a in range(3)]
        sg2 += sum(x * x for x in gr)
    gs2 = sum(x * x for x in g)
    scale = m / rho0
    denom = max(scale * scale * (sg2 + gs2) + eps, eps)
    if contrib < 2 or (sg2 + gs2) < 1e-12:
        return 0.0, dens, contrib
    lam = -(dens / rho0 - 1.0) / denom
    if abs(lam) > lam_max:
        lam = math.copysign(lam_max, lam)
    return lam, dens, contrib


def delta_of(i, pos, lam, order, kc, rho0, k, n, dqh, smin, omega, clamp_h):
    dq = dqh * kc["h"]
    wq = kc["poly6"] * (kc["h2"] - dq * dq) ** 3
    d = [0.0, 0.0, 0.0]
    for j in order[i]:
        if j == i:
            continue
        r = [pos[i][a] - pos[j][a] for a in range(3)]
        r2 = sum(x * x for x in r)
        if r2 > kc["h2"]:
            continue
        rr = math.sqrt(r2)
        coeff = -3.0 * kc["spiky"] * (kc["h"] - rr) ** 2 / max(rr, 1e-6)
        w = kc["poly6"] * (kc["h2"] - r2) ** 3
        sc = max(-k * (w / wq) ** n, smin)
        lij = lam[i] + lam[j] + sc
        d = [d[a] + lij * coeff * r[a] for a in range(3)]
    d = [x / rho0 * omega for x in d]
    md = clamp_h * kc["h"]
    l2 = sum(x * x for x in d)
    if l2 > md * md:
        s = md / (math.sqrt(l2) + 1e-20)
        d = [x * s for x in d]
    return d


def xsph_of(i, pos, vel, order, kc, m, rho0, c):
    s = [0.0, 0.0, 0.0]
    for j in order[i]:
        if j == i:
            continue
        r = [pos[i][a] - pos[j][a] for a in range(3)]
        r2 = sum(x * x for x in r)
        if r2 > kc["h2"]:
            continue
        w = kc["poly6"] * (kc["h2"] - r2) ** 3
        s = [s[a] + (vel[j][a] - vel[i][a]) * w for a in range(3)]
    return [vel[i][a] + c * (m / rho0) * s[a] for a in range(3)]


def f32(x):
    return struct.unpack("f", struct.pack("f", x))[0]


def case(name, pos, vel, h, m, rho0, eps, cap, lam_max=50.0):
    # FP64 arithmetic on the exact FP32 inputs the kernels see.
    pos = [[f32(x) for x in p] for p in pos]
    vel = [[f32(x) for x in v] for v in vel]
    h, m, rho0, eps, lam_max = f32(h), f32(m), f32(rho0), f32(eps), f32(lam_max)
    mins, maxs, cs = [0.0, 0.0, 0.0], [1.0, 1.0, 1.0], h
    dim = [int(math.ceil(1.0 / cs))] * 3
    kc = kernel(h)
    order, keys, sorted_ids = neighbour_order(pos, mins, cs, dim)
    lam, dens, contrib = [], [], []
    for i in range(len(pos)):
        a, b, c = lam_of(i, pos, order, kc, m, rho0, eps, cap, lam_max)
        lam.append(a)
        dens.append(b)
        contrib.append(c)
    delta = [delta_of(i, pos, lam, order, kc, rho0, 0.1, 4.0, 0.2, -0.25, 0.75, 0.05) for i in range(len(pos))]
    xs = [xsph_of(i, pos, vel, order, kc, m, rho0, 0.01) for i in range(len(pos))]
    return {
        "name": name,
        "params": {"h": h, "mass": m, "rest_density": rho0, "lambda_denom_eps": eps, "max_neighbors": cap,
                   "lambda_max_abs": lam_max, "scorr_k": 0.1, "scorr_n": 4.0, "scorr_dq_h": 0.2, "scorr_min": -0.25,
                   "relax_omega": 0.75, "disp_clamp_max_h": 0.05, "xsph_c": 0.01, "box": [mins, maxs],
                   "cell_size": cs, "dim": dim},
        "pos": pos,
        "vel": vel,
        "keys": keys,
        "sorted_ids": sorted_ids,
        "density": dens,
        "contrib": contrib,
        "lambda": lam,
        "delta": delta,
        "xsph_vel": xs,
    }


def main():
    cases = []
    # Three particles of one triangle inside one 0.1 cell: every particle has
    # two neighbours, so all lambdas are non-zero.
    cases.append(case("triangle_one_cell", [[0.51, 0.52, 0.53], [0.56, 0.52, 0.53], [0.535, 0.565, 0.53]],
                      [[0.1, 0.0, 0.0], [0.0, -0.2, 0.0], [0.0, 0.0, 0.3]], 0.1, 0.01, 1.0, 1e-4, 64))
    # A line of three across a cell boundary: the ends have one neighbour
    # (contrib < 2 -> lambda 0), the middle one has two (unequal distances).
    cases.append(case("line_across_cells", [[0.47, 0.55, 0.55], [0.53, 0.55, 0.55], [0.605, 0.55, 0.55]],
                      [[0.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, -1.0]], 0.1, 0.01, 1.0, 1e-4, 64))
    # Five particles, neighbour cap 2: the centre particle counts only the
    # first two neighbours in reference order.
    cases.append(case("neighbour_cap", [[0.55, 0.55, 0.55], [0.58, 0.55, 0.55], [0.52, 0.55, 0.55],
                                        [0.55, 0.58, 0.55], [0.55, 0.55, 0.61]],
                      [[0.0] * 3] * 5, 0.1, 0.01, 1.0, 1e-4, 2))
    # Lambda clamp: a tiny denominator makes |lambda| exceed lambda_max_abs.
    cases.append(case("lambda_clamp", [[0.51, 0.52, 0.53], [0.54, 0.52, 0.53], [0.525, 0.545, 0.53]],
                      [[0.0] * 3] * 3, 0.1, 1e-6, 1.0, 1e-12, 64, 5.0))
    with open(os.path.join(HERE, "kat_formulas.json"), "w") as f:
        json.dump(cases, f, indent=1)
    print("wrote", len(cases), "cases")


if __name__ == "__main__":
    main()
