"""Tolerances shared by the parity tests.

The plain FP32 GPU step must match the oracle within 1e-5 relative error. "Relative" is
taken against the natural scale of each quantity, because several outputs are small
differences of large terms:
  density      |d rho| <= tol * rho                   (all terms positive)
  pressure     |d p|   <= tol * k * rho               (p = k (rho - rho0) cancels)
  acceleration |d a|   <= tol * A, A = sum of the magnitudes of every force term / rho
                                    + |g| + wall terms (the oracle reports A per particle)
  position     |d x'|  <= 4 ulp(x') + tol * A * dt^2
  velocity     |d v'|  <= (4 ulp(x') + tol * A * dt^2) / dt   (v' = (x' - x) / dt)
"""
import numpy as np

TOL = 1e-5
K_GAS = 3.0
DT = 0.01


def ulp32(x):
    x = np.abs(np.asarray(x, np.float32))
    return np.spacing(np.maximum(x, np.float32(1e-30))).astype(np.float64)


def rel_errors(got, ref, k=K_GAS, dt=DT):
    """Per-quantity worst-case normalised errors (1.0 == exactly at the TOL bound)."""
    out = {}
    rho_r = np.asarray(ref["rho"], np.float64)
    if "rho" in got:
        out["rho"] = float(np.max(np.abs(np.asarray(got["rho"], np.float64) - rho_r) / (TOL * np.abs(rho_r))))
    if "p" in got:
        out["p"] = float(np.max(np.abs(np.asarray(got["p"], np.float64) - np.asarray(ref["p"], np.float64))
                                / (TOL * k * np.abs(rho_r))))
    A = np.asarray(ref["ascale"], np.float64)
    if "acc" in got:
        d = np.linalg.norm(np.asarray(got["acc"], np.float64) - np.asarray(ref["acc"], np.float64), axis=1)
        out["acc"] = float(np.max(d / (TOL * A)))
    if "pos" in got:
        bound = 4 * ulp32(ref["pos"]) + (TOL * A * dt * dt)[:, None]
        out["pos"] = float(np.max(np.abs(np.asarray(got["pos"], np.float64) - np.asarray(ref["pos"], np.float64))
                                  / bound))
    if "vel" in got:
        bound = (4 * ulp32(ref["pos"]) + (TOL * A * dt * dt)[:, None]) / dt
        out["vel"] = float(np.max(np.abs(np.asarray(got["vel"], np.float64) - np.asarray(ref["vel"], np.float64))
                                  / bound))
    return out


def assert_within(errs, what=""):
    bad = {k: v for k, v in errs.items() if not v <= 1.0}
    assert not bad, f"{what}: normalised errors above 1 (1 = tolerance {TOL}): {errs}"
