"""Scene generators of the library (host-only functions, no GPU) against numpy
restatements and the oracle's restatement of the reference's dam break."""
import math

import numpy as np
import pytest

H32 = np.float32(0.0457)
SPACING = np.float32(H32 / np.float32(2.0))
MASK64 = (1 << 64) - 1


class SplitMix64:
    def __init__(self, seed):
        self.s = seed & MASK64

    def next(self):
        self.s = (self.s + 0x9E3779B97F4A7C15) & MASK64
        z = self.s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
        return z ^ (z >> 31)

    def u24(self):
        return np.float32(self.next() >> 40) * np.float32(2.0 ** -24)

    def u53(self):
        return float(self.next() >> 11) * 2.0 ** -53


def lattice_numpy(box, dims, seed, jitter=0.01, spacing=SPACING):
    """Restatement of sph_scene_lattice: y outer, x, z inner; three jitter draws per particle."""
    rng = SplitMix64(seed)
    f = np.float32
    amp = f(f(jitter) * f(spacing))
    o = [f(-f(b) / f(2.0)) for b in box]
    n = int(np.prod(dims))
    out = np.zeros((n, 3), np.float32)
    k = 0
    for iy in range(dims[1]):
        for ix in range(dims[0]):
            for iz in range(dims[2]):
                j = [f(f(f(rng.u24() * f(2.0)) - f(1.0)) * amp) for _ in range(3)]
                out[k, 0] = f(f(o[0] + f(f(ix) * f(spacing))) + j[0])
                out[k, 1] = f(f(o[1] + f(f(iy) * f(spacing))) + j[1])
                out[k, 2] = f(f(o[2] + f(f(iz) * f(spacing))) + j[2])
                k += 1
    return out


@pytest.mark.parametrize("box", [0.1, 0.4, 0.7, 0.9, 1.0])
def test_reference_dam_break_matches_oracle(sphlib, oracle_mod, box):
    a = sphlib.reference_dam_break(box)
    b = oracle_mod.reference_dam_break(box)
    assert a.shape == b.shape
    assert np.array_equal(a, b)


@pytest.mark.parametrize("dims,box,seed", [((20, 20, 20), (1.0, 1.0, 0.5), 0), ((7, 3, 5), (0.5, 0.3, 0.4), 12345)])
def test_lattice_bit_exact(sphlib, dims, box, seed):
    got = sphlib.dam_break_scene(dims, box, seed)
    want = lattice_numpy(box, dims, seed)
    assert np.array_equal(got, want)
    # anchored at the min corner, within 1% of the spacing
    lo = -np.asarray(box, np.float32) / 2
    assert np.all(got.min(axis=0) >= lo - 0.0101 * SPACING)
    assert np.all(got.min(axis=0) <= lo + 0.0101 * SPACING)


@pytest.mark.parametrize("dims,box,seed", [((20, 20, 20), (1.0, 1.0, 0.5), 0), ((7, 3, 5), (0.5, 0.3, 0.4), 12345),
                                            ((100, 100, 100), (5.0, 5.0, 2.5), 1)])
def test_oracle_lattice_equals_library_lattice(sphlib, dims, box, seed):
    """The oracle's vectorised restatement (the reference arm's input, built without the
    product library) gives the library generator's coordinates bit for bit, up to the 1M scene."""
    from oracle import scenes

    assert np.array_equal(scenes.dam_break(dims, box, seed), sphlib.dam_break_scene(dims, box, seed))


def test_batch_plan(sphlib):
    dims, boxes = sphlib.batch_plan(256, seed=3)
    rng = SplitMix64(3)
    for s in range(256):
        nt = math.exp(math.log(2000) + rng.u53() * (math.log(64000) - math.log(2000)))
        a = [0.5 + rng.u53() * 1.5 for _ in range(3)]
        base = (nt / (a[0] * a[1] * a[2])) ** (1.0 / 3.0)
        d = [max(1, int(math.floor(base * a[k] + 0.5))) for k in range(3)]
        assert list(dims[s]) == d
        per = (1 / 20, 1 / 20, 0.5 / 20)
        np.testing.assert_array_equal(boxes[s], np.array([d[k] * per[k] for k in range(3)], np.float32))
    n = dims.prod(axis=1)
    assert 1500 <= n.min() and n.max() <= 80000
    assert 3.0e6 < n.sum() < 7.0e6


def test_fountain_emitter(sphlib):
    xyz, vel = sphlib.fountain_emit(seed=2, step=5, n=2000, center=(0.0, -0.99, 0.0), radius=0.05, speed=5.0,
                                    sigma=0.2)
    xyz2, vel2 = sphlib.fountain_emit(seed=2, step=5, n=2000, center=(0.0, -0.99, 0.0), radius=0.05, speed=5.0,
                                      sigma=0.2)
    assert np.array_equal(xyz, xyz2) and np.array_equal(vel, vel2)
    r = np.hypot(xyz[:, 0], xyz[:, 2])
    assert r.max() <= 0.05 + 1e-6
    assert np.all(xyz[:, 1] == np.float32(-0.99))
    assert abs(vel[:, 1].mean() - 5.0) < 0.03 and abs(vel[:, 0].std() - 0.2) < 0.02
    x3, _ = sphlib.fountain_emit(seed=2, step=6, n=2000, center=(0.0, -0.99, 0.0), radius=0.05, speed=5.0, sigma=0.2)
    assert not np.array_equal(xyz, x3)


def test_fountain_emitter_distribution(sphlib):
    """The emitter's normals (Marsaglia's polar method with the generator's own logarithm) and
    its disc sampling have the stated distribution."""
    n = 200000
    xyz, vel = sphlib.fountain_emit(seed=9, step=0, n=n, center=(0.0, 0.0, 0.0), radius=1.0, speed=0.0, sigma=1.0)
    g = vel.astype(np.float64)
    assert np.all(np.abs(g.mean(axis=0)) < 0.01)
    assert np.all(np.abs(g.std(axis=0) - 1.0) < 0.01)
    # fourth moment of a normal is 3 (standard error 0.022 at this n); the tails are present
    assert np.all(np.abs((g ** 4).mean(axis=0) - 3.0) < 0.1)
    assert np.all(np.abs(g).max(axis=0) > 4.0)
    stats = pytest.importorskip("scipy.stats")
    for a in range(3):
        assert stats.kstest(g[:, a], "norm").pvalue > 1e-4
    r2 = xyz[:, 0].astype(np.float64) ** 2 + xyz[:, 2].astype(np.float64) ** 2
    assert r2.max() <= 1.0 + 1e-6
    # uniform on the disc: P(r^2 < t) = t
    for t in (0.1, 0.25, 0.5, 0.9):
        assert abs(np.mean(r2 < t) - t) < 0.005
    # particles of one step are independent of how many are drawn
    x2, v2 = sphlib.fountain_emit(seed=9, step=0, n=100, center=(0.0, 0.0, 0.0), radius=1.0, speed=0.0, sigma=1.0)
    assert np.array_equal(x2, xyz[:100]) and np.array_equal(v2, vel[:100])
