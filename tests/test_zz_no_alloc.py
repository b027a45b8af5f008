"""pimc_adjoint_noalloc: the adjoint with its scratch in static device memory.

Called through the C ABI and compared with pimc_adjoint on the same chain,
twice in a row (the first call on the device does the set-up, the second
reuses it).  The file is collected last so that it also runs after every
other test of the session; it passes alone in a fresh process as well.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _adjoint(e, fn, chain, dim, N, M):
    g, th, ex = np.zeros((dim, N, M)), np.zeros(3), np.zeros(4)
    rc = fn(e.h, chain, _dp(g), _dp(th), _dp(ex))
    return rc, g, th, ex


def _chain(**kw):
    from pimc.engine import ChainParams
    base = dict(dim=2, L=6.0, T=0.5, lam=0.5, harmonic_omega=0.7, lattice_V0=2.0, lattice_a=1.0,
                interactions=True, pair_g=1.0, pair_sigma=0.5, r_a=1.2, semantics=1, seed=5)
    base.update(kw)
    return ChainParams(**base)


def test_noalloc_adjoint_matches_allocating_adjoint_twice():
    from pimc.engine import Engine
    chains = [_chain(N=24, M=16, seed=5), _chain(N=40, M=32, seed=6)]
    e = Engine(chains)
    rng = np.random.default_rng(21)
    for c, p in enumerate(chains):
        e.set_beads(rng.normal(scale=1.2, size=(p.dim, p.N, p.M)), chain=c)
    e.run_batched(3)  # some accepted moves, permuted cycles
    L = e.L
    for c, p in enumerate(chains):
        rc, g0, th0, ex0 = _adjoint(e, L.pimc_adjoint, c, p.dim, p.N, p.M)
        assert rc == 0, L.pimc_last_error()
        for _ in range(2):
            rc, g1, th1, ex1 = _adjoint(e, L.pimc_adjoint_noalloc, c, p.dim, p.N, p.M)
            assert rc == 0, L.pimc_last_error()
            np.testing.assert_allclose(g1, g0, rtol=RTOL, atol=1e-300)
            np.testing.assert_allclose(th1, th0, rtol=RTOL, atol=1e-300)
            np.testing.assert_allclose(ex1, ex0, rtol=RTOL, atol=1e-300)
            assert np.any(g1 != 0.0)
    e.close()


def test_noalloc_adjoint_refuses_chains_above_its_limit():
    from pimc.engine import Engine
    p = _chain(N=700, M=100, interactions=False)  # 70000 beads > 65536
    e = Engine([p])
    rc, _, _, _ = _adjoint(e, e.L.pimc_adjoint_noalloc, 0, p.dim, p.N, p.M)
    assert rc != 0
    assert b"65536" in e.L.pimc_last_error()
    # the allocating entry point still serves it
    rc, g, _, _ = _adjoint(e, e.L.pimc_adjoint, 0, p.dim, p.N, p.M)
    assert rc == 0 and np.all(np.isfinite(g))
    e.close()
