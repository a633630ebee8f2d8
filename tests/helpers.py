"""Shared test helpers: seeded random states/unitaries and tolerance checks.

Tolerances follow the parity bar for this path: 1e-12 for complex128 and 1e-5
for complex64 (absolute on normalized states, relative with an absolute floor
for expectation values and Jacobian entries, which can be exactly zero).
"""
import zlib

import numpy as np

TOL = {np.complex128: 1e-12, np.complex64: 1e-5}
DTYPES = [np.complex128, np.complex64]


def tol_of(dt) -> float:
    return TOL[np.dtype(dt).type]


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


def assert_close(a, b, dt, scale=1.0, what=""):
    a = np.asarray(a)
    b = np.asarray(b)
    t = tol_of(dt) * scale
    err = np.max(np.abs(a - b)) if a.size else 0.0
    ref = max(1.0, float(np.max(np.abs(b))) if b.size else 1.0)
    assert err <= t * ref, f"{what}: max|diff| = {err:.3e} > {t * ref:.3e}"


def sv_class(ops, dt):
    return ops.StateVectorC128 if np.dtype(dt) == np.complex128 else ops.StateVectorC64


def meas_class(ops, dt):
    return ops.MeasurementsC128 if np.dtype(dt) == np.complex128 else ops.MeasurementsC64


def obs_ns(ops, dt):
    suffix = "C128" if np.dtype(dt) == np.complex128 else "C64"
    o = ops.observables
    return (getattr(o, "NamedObs" + suffix), getattr(o, "HermitianObs" + suffix), getattr(o, "TensorProdObs" + suffix),
            getattr(o, "Hamiltonian" + suffix), getattr(o, "SparseHamiltonian" + suffix))
