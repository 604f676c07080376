"""Generates ref_cl_cases.npz: outputs of the reference's own OpenCL grid kernels
(resources/kernels/sph_grid.cl density_pressure_step and forces_step, compiled for the CPU by
oracle/ref_cl where the reference tree is present) on a few states, for the GPU parity tests
on machines without the reference tree.

    python tests/golden/make_ref_cl_golden.py

Each case: a box, gravity, a state (positions, velocities) reached by stepping the oracle
from a seeded scene, and the kernels' density, pressure and acceleration (before the walls);
for the 0.4 m dam break also those of the all-pairs kernels (sph_brute.cl).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "gmu-water-simulation_gb300"))

from oracle import oracle as O  # noqa: E402

OUT = os.path.join(HERE, "ref_cl_cases.npz")

# (name, box, gravity, scene, oracle steps before the evaluation)
CASES = [
    ("dam0.4_step0", (0.4, 0.4, 0.4), (0.0, -9.80665, 0.0), "reference", 0),
    ("dam0.4_step40", (0.4, 0.4, 0.4), (0.0, -9.80665, 0.0), "reference", 40),
    ("lattice16_step15", (1.0, 1.0, 0.5), (0.0, -9.81, 0.0), "lattice16", 15),
]


def scene(kind):
    if kind == "reference":
        return O.reference_dam_break(0.4)
    import sphcuda

    return sphcuda.dam_break_scene((16, 16, 16), (1.0, 1.0, 0.5), 3)


def main():
    O.build()
    root = os.environ.get("SPH_REFERENCE_ROOT", "/root/reference")  # the reference tree
    if O.build_ref(os.path.join(root, "resources", "kernels")) is None:
        raise SystemExit("the reference tree is not present: nothing to generate")
    out = {}
    for name, box, g, kind, steps in CASES:
        o = O.Oracle(box, O.REF, threads=4, gravity=g)
        o.add(scene(kind))
        o.step(steps)
        st = o.state()
        rho, p, acc = O.ref_density_forces(st["pos"], st["vel"], box, g)
        out[name + "/box"] = np.asarray(box, np.float32)
        out[name + "/gravity"] = np.asarray(g, np.float32)
        out[name + "/pos"] = st["pos"]
        out[name + "/vel"] = st["vel"]
        out[name + "/rho"] = rho
        out[name + "/p"] = p
        out[name + "/acc"] = acc
        if kind == "reference":  # the all-pairs kernels (sph_brute.cl) on the small scenes
            rb, pb, ab = O.ref_brute_density_forces(st["pos"], st["vel"], g)
            out[name + "/brute_rho"] = rb
            out[name + "/brute_p"] = pb
            out[name + "/brute_acc"] = ab
    np.savez_compressed(OUT, names=np.array([c[0] for c in CASES]), **out)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
