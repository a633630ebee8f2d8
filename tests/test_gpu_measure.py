"""GPU measurements vs the CPU oracle: probs (index ordering), expval / var of
named, Hermitian, Pauli-sum, mixed and sparse observables, seeded samples.

Mirrors pennylane_lightning/core/simulators/lightning_qubit/measurements/tests/
Test_MeasurementsLQubit.cpp (:205-430 expval by name/matrix, :534-968 probs
index ordering with permuted targets) and core/measurements/tests/
Test_MeasurementsBase.cpp (:1319-1323 seeded samples); Metropolis-Hastings
samples (MeasurementsLQubit.hpp:551-594, TransitionKernels.hpp) exactly as
the oracle draws them.
"""
import numpy as np
import pytest

from helpers import DTYPES, assert_close, assert_scalar, meas_class, obs_ns, rand_hermitian, rand_state, seed_of, sv_class

pytestmark = pytest.mark.gpu

WIRE_LISTS = [None, [0], [6], [2, 5], [5, 2], [1, 4, 6], [6, 0, 3, 2], [0, 1, 2, 3, 4], [4, 2, 0, 6, 5, 1],
              [0, 1, 2, 3, 4, 5, 6], [6, 5, 4, 3, 2, 1, 0]]


def _setup(ops, oracle, n, dt, seed):
    rng = np.random.default_rng(seed)
    st = rand_state(rng, n, dt)
    sv = sv_class(ops, dt)(n)
    sv.updateData(st)
    o = oracle.sv(n, dt)
    o.set_state(st)
    return rng, sv, meas_class(ops, dt)(sv), o


@pytest.mark.parametrize("dt", DTYPES)
def test_probs_ordering(ops_module, oracle, dt):
    _, sv, m, o = _setup(ops_module, oracle, 7, dt, seed_of("probs", dt.__name__))
    # the all-wires distribution is element-wise and every marginal is
    # summed in the reference's order: bit-exact, in the output order the
    # wire list gives
    for wires in WIRE_LISTS:
        p = m.probs() if wires is None else m.probs(wires)
        assert np.array_equal(np.asarray(p, np.float64), o.probs(wires)), wires


@pytest.mark.parametrize("dt", DTYPES)
def test_expval_var_named(ops_module, oracle, dt):
    _, sv, m, o = _setup(ops_module, oracle, 6, dt, seed_of("named", dt.__name__))
    for name in ("PauliX", "PauliY", "PauliZ", "Hadamard", "Identity"):
        for w in range(6):
            # a one-wire observable has norm 1: its expval / var errors are
            # relative to 1 (both can be exactly 0 for Identity)
            assert_scalar(m.expval(name, [w]), o.expval_named(name, [w]), dt, mag=1.0, what=f"E {name}{w}")
            assert_scalar(m.var(name, [w]), o.var_named(name, [w]), dt, mag=1.0, what=f"V {name}{w}")


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("k", [1, 2, 3, 4, 5, 6])
def test_expval_var_matrix(ops_module, oracle, k, dt):
    rng, sv, m, o = _setup(ops_module, oracle, 8, dt, seed_of("hmat", k, dt.__name__))
    H = rand_hermitian(rng, k)
    w = [int(x) for x in rng.choice(8, size=k, replace=False)]
    # errors of <H> and var(H) = <H^2> - <H>^2 scale with ||H|| and ||H||^2
    hn = float(np.linalg.norm(H, 2))
    assert_scalar(m.expval(H, w), o.expval_matrix(H, w), dt, mag=hn, what="E herm")
    assert_scalar(m.var(H, w), o.var_matrix(H, w), dt, mag=hn * hn, what="V herm")


def _pauli_terms(rng, n, nterms, maxw=4):
    terms = []
    for _ in range(nterms):
        wt = int(rng.integers(1, maxw + 1))
        terms.append((float(rng.normal()), "".join(rng.choice(list("XYZ"), size=wt)),
                      [int(x) for x in rng.choice(n, size=wt, replace=False)]))
    return terms


def _ham_obs(ops, dt, terms):
    Named, Herm, Prod, Ham, _ = obs_ns(ops, dt)
    names = {"X": "PauliX", "Y": "PauliY", "Z": "PauliZ"}
    return Ham([c for c, _, _ in terms],
               [Prod([Named(names[ch], [w]) for ch, w in zip(word, wires)]) for _, word, wires in terms])


@pytest.mark.parametrize("dt", DTYPES)
def test_expval_pauli_hamiltonian(ops_module, oracle, dt):
    from oracle.pyoracle import pauli_sum_spec

    rng, sv, m, o = _setup(ops_module, oracle, 10, dt, seed_of("ham", dt.__name__))
    terms = _pauli_terms(rng, 10, 64)
    # repeated flip masks: same X/Y positions, different Z tails
    terms += [(0.5, "XZ", [1, 4]), (-0.25, "XZ", [1, 7]), (0.75, "YY", [2, 3]), (0.1, "XX", [2, 3])]
    H = _ham_obs(ops_module, dt, terms)
    spec = pauli_sum_spec(terms)
    # the error of a Pauli-sum expectation is relative to sum |c| (each word
    # has norm 1), that of the variance to (sum |c|)^2
    c1 = sum(abs(t[0]) for t in terms)
    assert_scalar(m.expval(H), o.expval_obs(spec), dt, mag=c1, what="E ham")
    assert_scalar(m.var(H), o.var_obs(spec), dt, mag=c1 * c1, what="V ham")


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("n", [12, 15])
def test_expval_pauli_hamiltonian_tiles(ops_module, oracle, dt, n):
    # registers of 12 or more qubits: words evaluated in passes over tiles of
    # 2^12 amplitudes (the pipelined pass kernel) -- diagonal words, Re and
    # Im words (even / odd Y count), repeated flip masks, words of high weight
    # -- and words with more flip bits than a tile holds (one sweep per mask)
    from oracle.pyoracle import pauli_sum_spec

    rng, sv, m, o = _setup(ops_module, oracle, n, dt, seed_of("ham-tiles", dt.__name__, n))
    terms = _pauli_terms(rng, n, 48) + _pauli_terms(rng, n, 16, maxw=8)
    terms += [(0.5, "XZ", [1, 4]), (-0.25, "XZ", [1, 7]), (0.75, "YY", [2, 3]), (0.1, "XX", [2, 3]),
              (0.3, "Y", [n - 1]), (-0.6, "ZZ", [0, n - 1]), (0.2, "Z", [5])]
    wide = list(range(n - 1))  # 11 or 14 flip bits
    terms += [(0.4, ("XY" * n)[: len(wide)], wide), (-0.35, ("YYX" * n)[: len(wide)] + "Z", wide + [n - 1])]
    H = _ham_obs(ops_module, dt, terms)
    spec = pauli_sum_spec(terms)
    c1 = sum(abs(t[0]) for t in terms)
    assert_scalar(m.expval(H), o.expval_obs(spec), dt, mag=c1, what=f"E ham {n}q")


@pytest.mark.parametrize("dt", DTYPES)
def test_expval_mixed_observables(ops_module, oracle, dt):
    from oracle.pyoracle import ObsData

    rng, sv, m, o = _setup(ops_module, oracle, 7, dt, seed_of("mixed", dt.__name__))
    Named, Herm, Prod, Ham, _ = obs_ns(ops_module, dt)
    H2 = rand_hermitian(rng, 2)
    od = ObsData()
    off = od.add_matrix(H2)
    obs = Ham([0.5, -1.25, 0.3],
              [Prod([Named("PauliX", [0]), Herm(H2, [3, 5])]), Named("PauliY", [2]),
               Prod([Named("Hadamard", [1]), Named("PauliZ", [6])])])
    spec = (f"ham 3 0.5 prod 2 named PauliX 0 herm 2 3 5 {off} -1.25 named PauliY 2 "
            f"0.3 prod 2 named Hadamard 1 named PauliZ 6")
    c1 = 0.5 * float(np.linalg.norm(H2, 2)) + 1.25 + 0.3  # sum of |c| x term norms
    assert_scalar(m.expval(obs), o.expval_obs(spec, od), dt, mag=c1, what="E mixed")
    assert_scalar(m.var(obs), o.var_obs(spec, od), dt, mag=c1 * c1, what="V mixed")
    single = Prod([Named("PauliZ", [0]), Named("PauliZ", [1]), Named("PauliZ", [2])])
    assert_scalar(m.expval(single), o.expval_obs("prod 3 named PauliZ 0 named PauliZ 1 named PauliZ 2"), dt,
                  mag=1.0, what="E ZZZ")


@pytest.mark.parametrize("dt", DTYPES)
def test_expval_sparse(ops_module, oracle, dt):
    import scipy.sparse as sp

    rng, sv, m, o = _setup(ops_module, oracle, 7, dt, seed_of("sp", dt.__name__))
    A = sp.random(128, 128, density=0.05, random_state=3) + 1j * sp.random(128, 128, density=0.05, random_state=4)
    A = (A + A.conj().T).tocsr()
    A.sort_indices()
    an = float(np.linalg.norm(A.toarray(), 2))
    assert_scalar(m.expval(A.indptr, A.indices, A.data), o.expval_sparse(A.indptr, A.indices, A.data), dt,
                  mag=an, what="E sparse")
    *_, Sparse = obs_ns(ops_module, dt)
    obs = Sparse(A.data, A.indices, A.indptr, list(range(7)))
    assert_scalar(m.expval(obs), o.expval_sparse(A.indptr, A.indices, A.data), dt, mag=an, what="E sparseH")


@pytest.mark.parametrize("dt", DTYPES)
def test_samples_exact(ops_module, oracle, dt):
    # Integer outputs under a fixed seed must be identical to the oracle's.
    _, sv, m, o = _setup(ops_module, oracle, 8, dt, seed_of("samples", dt.__name__))
    m.set_random_seed(37)
    s = m.generate_samples(8, 5000)
    assert s.shape == (5000, 8)
    assert np.array_equal(s.astype(np.int64), o.samples(5000, 37))
    for wires in ([3], [7, 0, 2]):
        s = m.generate_samples(wires, 3000)
        assert np.array_equal(s.astype(np.int64), o.samples(3000, 37, wires))


@pytest.mark.parametrize("dt", DTYPES)
def test_mcmc_samples_exact(ops_module, oracle, dt):
    # generate_mcmc_samples: both transition-kernel names, with and without
    # burn-in, on a dense state and on one with zero amplitudes (which the
    # non-zero-random kernel never proposes).  Integer outputs must equal the
    # oracle's for the same seed.
    rng, sv, m, o = _setup(ops_module, oracle, 9, dt, seed_of("mcmc", dt.__name__))
    for zeros in (False, True):
        if zeros:
            st = rand_state(rng, 9, dt)
            st[rng.random(st.size) < 0.5] = 0
            st = (st / np.linalg.norm(st)).astype(dt)
            sv.updateData(st)
            o.set_state(st)
        for kname in ("Local", "NonZeroRandom"):
            for burnin, shots, seed in ((0, 4000, 3), (250, 3000, 77)):
                m.set_random_seed(seed)
                s = m.generate_mcmc_samples(9, kname, burnin, shots)
                assert s.shape == (shots, 9)
                assert np.array_equal(s.astype(np.int64), o.mcmc_samples(kname, burnin, shots, seed)), (zeros, kname)


@pytest.mark.parametrize("dt", DTYPES)
def test_mcmc_samples_large_register(ops_module, oracle, dt):
    # 2^20 amplitudes: 256 counting chunks, so the rank -> index search spans
    # chunk boundaries.
    rng, sv, m, o = _setup(ops_module, oracle, 20, dt, seed_of("mcmc20", dt.__name__))
    m.set_random_seed(2024)
    s = m.generate_mcmc_samples(20, "Local", 100, 2000)
    assert np.array_equal(s.astype(np.int64), o.mcmc_samples("Local", 100, 2000, 2024))


@pytest.mark.parametrize("dt", DTYPES)
def test_mcmc_samples_edges(ops_module, oracle, dt):
    from lightning_gb300.lightning_gb300_ops import LightningException

    rng, sv, m, o = _setup(ops_module, oracle, 4, dt, seed_of("mcmc-edge", dt.__name__))
    m.set_random_seed(1)
    assert m.generate_mcmc_samples(4, "Local", 10, 0).shape == (0, 4)
    with pytest.raises(LightningException):
        m.generate_mcmc_samples(3, "Local", 0, 10)  # every qubit is sampled
    sv.updateData(np.zeros(16, dtype=dt))
    with pytest.raises(LightningException):
        m.generate_mcmc_samples(4, "Local", 0, 10)  # no non-zero amplitude to propose


@pytest.mark.parametrize("dt", DTYPES)
def test_large_pauli_sum_apply_chunks(ops_module, oracle, dt):
    # var of a Pauli sum with more flip-mask groups than one launch of the
    # one-sweep application takes (256): the application runs in chunks, the
    # later ones adding to the first's output.
    from oracle.pyoracle import pauli_sum_spec

    rng, sv, m, o = _setup(ops_module, oracle, 10, dt, seed_of("bigham", dt.__name__))
    terms = []
    seen = set()
    while len(terms) < 400:
        k = int(rng.integers(1, 5))
        wires = [int(x) for x in rng.choice(10, size=k, replace=False)]
        word = "".join(rng.choice(list("XYZ"), size=k))
        key = (word, tuple(wires))
        if key in seen:
            continue
        seen.add(key)
        terms.append((float(rng.normal()), word, wires))
    Named, _, Prod, Ham, _ = obs_ns(ops_module, dt)
    H = Ham([t[0] for t in terms], [Prod([Named("Pauli" + c, [w]) for c, w in zip(t[1], t[2])]) for t in terms])
    spec = pauli_sum_spec(terms)
    c1 = sum(abs(t[0]) for t in terms)
    assert_scalar(m.expval(H), o.expval_obs(spec), dt, mag=c1, what="E big H")
    assert_scalar(m.var(H), o.var_obs(spec), dt, mag=c1 * c1, what="var big H")
