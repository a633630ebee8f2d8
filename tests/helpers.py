"""Shared test helpers: seeded random states/unitaries and the parity checks.

The parity bar for this path is 1e-12 relative for complex128 and 1e-5
relative for complex64.  The checks apply it without multipliers:

* states (``assert_state``): norm-relative ``||a - b|| / ||b|| <= tol`` and
  per-amplitude relative ``|a_i - b_i| / |b_i| <= tol`` wherever
  ``|b_i| >= tau * max|b|``.  The floor tau exists because two exact-FP64
  evaluations of one circuit in different orders already differ by more than
  1e-12 relative on the smallest amplitudes: the config-1 circuit (20 cycles
  of Haar SU(2) + CZ) at 22 qubits, applied gate by gate by the oracle and
  by numpy tensordot, differs by 2.3e-15 norm-relative but by 1.2e-11
  relative on amplitudes at 1e-6 * max, 9.2e-13 at 1e-3 * max and 1.5e-13 at
  1e-2 * max.  Rounding errors are absolute (a fraction of the norm), so the
  relative error of an amplitude grows as its size falls.  tau = 1e-2 for
  complex128 (every amplitude but the smallest ~0.2 %); 1e-1 for complex64,
  whose 2^-24 rounding is 2^29 times larger;
* vectors of results (Jacobians, expectation-value lists, probabilities):
  the same two checks with the same tau;
* scalars (``assert_scalar``): ``|a - b| <= tol * max(|b|, mag)`` where
  ``mag`` names the quantity's natural size when it can cancel to near zero
  (a variance E[O^2] - E[O]^2 is computed by the reference, and here, as a
  difference, so its error is relative to E[O^2]); mag defaults to 0, which
  makes the check purely relative.
"""
import zlib

import numpy as np

TOL = {np.complex128: 1e-12, np.complex64: 1e-5}
TAU = {np.complex128: 1e-2, np.complex64: 1e-1}
DTYPES = [np.complex128, np.complex64]


def tol_of(dt) -> float:
    return TOL[np.dtype(dt).type]


def tau_of(dt) -> float:
    return TAU[np.dtype(dt).type]


def seed_of(*parts) -> int:
    return zlib.crc32("/".join(map(str, parts)).encode())


def rand_state(rng, n, dt=np.complex128):
    v = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    v /= np.linalg.norm(v)
    return v.astype(dt)


def rand_unitary(rng, k):
    d = 1 << k
    m = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    q, r = np.linalg.qr(m)
    return q * (np.diag(r) / np.abs(np.diag(r)))


def rand_hermitian(rng, k):
    d = 1 << k
    m = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    return (m + m.conj().T) / 2


def rel_errors(a, b, dt):
    """(norm-relative error, max per-element relative error over |b_i| >=
    tau * max|b|) of a against the reference b."""
    a = np.asarray(a, dtype=np.complex128).ravel()
    b = np.asarray(b, dtype=np.complex128).ravel()
    nb = float(np.linalg.norm(b))
    if nb == 0.0:
        return float(np.linalg.norm(a)), 0.0
    nr = float(np.linalg.norm(a - b)) / nb
    mag = np.abs(b)
    sel = mag >= tau_of(dt) * mag.max()
    pr = float(np.max(np.abs(a[sel] - b[sel]) / mag[sel])) if sel.any() else 0.0
    return nr, pr


def assert_state(a, b, dt, what=""):
    """States and result vectors: norm-relative and per-element relative."""
    assert np.asarray(a).shape == np.asarray(b).shape, f"{what}: shape {np.shape(a)} != {np.shape(b)}"
    if np.asarray(b).size == 0:
        return
    t = tol_of(dt)
    nr, pr = rel_errors(a, b, dt)
    assert nr <= t, f"{what}: norm-relative error {nr:.3e} > {t:.1e}"
    assert pr <= t, f"{what}: per-element relative error {pr:.3e} > {t:.1e} (|b_i| >= {tau_of(dt):g} max|b|)"


# states and vectors use the same check
assert_close = assert_state


def assert_scalar(a, b, dt, mag=0.0, what=""):
    """Scalars: relative to max(|b|, mag) (mag: the natural size of a
    quantity that can cancel, e.g. E[O^2] for a variance)."""
    t = tol_of(dt)
    a, b = complex(a), complex(b)
    den = max(abs(b), float(mag))
    err = abs(a - b)
    assert err <= t * den, f"{what}: |a - b| = {err:.3e} > {t:.1e} x {den:.3e}"


def sv_class(ops, dt):
    return ops.StateVectorC128 if np.dtype(dt) == np.complex128 else ops.StateVectorC64


def meas_class(ops, dt):
    return ops.MeasurementsC128 if np.dtype(dt) == np.complex128 else ops.MeasurementsC64


def obs_ns(ops, dt):
    suffix = "C128" if np.dtype(dt) == np.complex128 else "C64"
    o = ops.observables
    return (getattr(o, "NamedObs" + suffix), getattr(o, "HermitianObs" + suffix), getattr(o, "TensorProdObs" + suffix),
            getattr(o, "Hamiltonian" + suffix), getattr(o, "SparseHamiltonian" + suffix))
