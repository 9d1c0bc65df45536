"""Pin the CPU oracle against the L2/Linf goldens of Trixi.jl's own regression tests.

Each case reruns a TreeMesh Euler elixir (settings in tests/golden/trixi_goldens.json,
extracted from test/test_tree_{2,3}d_euler.jl) with the oracle's restatement of
Trixi's DGSEM rhs!, its 2N54 integrator and StepsizeCallback, and compares the
final error norms.  Trixi's tests use rtol = sqrt(eps); the oracle is held to 1e-9.
"""
import numpy as np
import pytest

from _cases import ic_id, load_goldens, oracle_from_case

GOLDENS = load_goldens()


@pytest.mark.parametrize("name", sorted(GOLDENS))
def test_oracle_reproduces_trixi_golden(oracle_mod, name):
    O = oracle_mod
    c = GOLDENS[name]
    orc = oracle_from_case(O, c)
    ic = ic_id(O, c["ic"])
    par = c.get("ic_params")
    u0 = orc.initial_condition(ic, par, c["tspan"][0])
    u, t, nsteps = orc.solve(u0, c["tspan"][0], c["tspan"][1], c["cfl"],
                             max_steps=c.get("maxiters", 10**9))
    l2, linf = orc.error_norms(u, t, ic, par)
    if "maxiters" in c:
        # free-stream preservation: goldens are round-off (~1e-16); compare absolutely
        assert np.all(l2 < 1e-14) and np.all(linf < 1e-13)
        assert np.allclose(l2, c["l2"], atol=5e-15, rtol=0)
        return
    assert t == pytest.approx(c["tspan"][1], rel=1e-14)
    np.testing.assert_allclose(l2, c["l2"], rtol=1e-9, atol=0)
    np.testing.assert_allclose(linf, c["linf"], rtol=1e-8, atol=0)
