"""Seeded synthetic scenes for the oracle, restated in numpy (test infrastructure only).

The reference arm of the benchmark and the tests build their dam-break inputs here, so
that timing the oracle never loads the product library. The generator is the product's
jittered lattice (sph_scene_lattice in the product's scene generators), restated so that
both give the same coordinates bit for bit:

  splitmix64 (Steele, Lea and Flood, 2014): the k-th output of a generator seeded with s is
  mix(s + k * 0x9E3779B97F4A7C15 mod 2^64), k = 1, 2, ...; a uniform draw in [0, 1) is the
  top 24 bits times 2^-24 (exact in float32).
  Particles are laid out y outer, then x, then z; each takes three draws (x, y, z jitter),
  jitter = (2 u - 1) * (jitter_fraction * spacing), coordinate = (-box/2 + i * spacing) + jitter,
  every operation rounded to float32 in that order.

The reference's own dam break (src/CBaseParticleSimulator.cpp:38-58) is restated in
sph_oracle.c (orc_reference_dam_break).
"""
import numpy as np

GAMMA = np.uint64(0x9E3779B97F4A7C15)
H32 = np.float32(0.0457)  # include/CParticle.h:80
SPACING = np.float32(H32 / np.float32(2.0))


def splitmix64(seed, count):
    """The first `count` outputs of splitmix64 seeded with `seed` (uint64 array)."""
    with np.errstate(over="ignore"):
        k = np.arange(1, count + 1, dtype=np.uint64)
        z = np.uint64(seed) + k * GAMMA
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def lattice(dims, box, seed, jitter=0.01, spacing=SPACING):
    """Jittered lattice of dims[0] x dims[1] x dims[2] particles anchored at the box's min
    corner, in the generator's id order (float32, shape (n, 3))."""
    f = np.float32
    dx, dy, dz = (int(d) for d in dims)
    n = dx * dy * dz
    u = (splitmix64(seed, 3 * n) >> np.uint64(40)).astype(f) * f(2.0 ** -24)
    amp = f(f(jitter) * f(spacing))
    j = ((u * f(2.0)) - f(1.0)) * amp
    j = j.reshape(n, 3)
    iy, ix, iz = np.meshgrid(np.arange(dy), np.arange(dx), np.arange(dz), indexing="ij")
    idx = [ix.reshape(-1), iy.reshape(-1), iz.reshape(-1)]
    out = np.empty((n, 3), f)
    for a in range(3):
        o = f(-f(box[a]) / f(2.0))
        out[:, a] = (o + idx[a].astype(f) * f(spacing)) + j[:, a]
    return out


def dam_break(dims, box, seed):
    """The synthetic dam breaks: a lattice at 0.5 h spacing with +-1% jitter."""
    return lattice(dims, box, seed)
