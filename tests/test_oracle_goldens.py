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
    if c.get("amr"):
        u, t, nsteps = orc.solve_amr(ic, par, c["tspan"][0], c["tspan"][1], c["cfl"],
                                     max_steps=c.get("maxiters", 10**9))
    else:
        u0 = orc.initial_condition(ic, par, c["tspan"][0])
        u, t, nsteps = orc.solve(u0, c["tspan"][0], c["tspan"][1], c["cfl"],
                                 max_steps=c.get("maxiters", 10**9))
    l2, linf = orc.error_norms(u, t, ic, par)
    if c["ic"] == "constant":
        # free-stream preservation: goldens are round-off (~1e-16); compare absolutely
        assert np.all(l2 < 1e-14) and np.all(linf < 1e-13)
        assert np.allclose(l2, c["l2"], atol=5e-15, rtol=0)
        return
    if "maxiters" in c:
        assert nsteps == c["maxiters"]
    else:
        assert t == pytest.approx(c["tspan"][1], rel=1e-14)
    np.testing.assert_allclose(l2, c["l2"], rtol=1e-9, atol=0)
    np.testing.assert_allclose(linf, c["linf"], rtol=1e-8, atol=0)


def test_oracle_entropy_timederivative_ec_vs_llf():
    # analysis_dg2d.jl:460-472 on a perturbed weak blast wave: zero up to rounding for
    # the entropy-conservative flux_ranocha surface flux, negative for LLF
    from oracle import oracle as O
    kw = dict(volume_integral=O.VI_FLUXDIFF, volume_flux=O.FLUX_RANOCHA)
    ec = O.Oracle(2, 3, 3, [-2.0, -2.0], [2.0, 2.0], surface_flux=O.FLUX_RANOCHA, **kw)
    llf = O.Oracle(2, 3, 3, [-2.0, -2.0], [2.0, 2.0], surface_flux=O.FLUX_LAX_FRIEDRICHS, **kw)
    u = ec.initial_condition(O.IC_WEAK_BLAST_WAVE)
    # nodal interpolation is continuous across interfaces; a perturbation
    # opens jumps for the surface flux to act on
    u *= 1.0 + 0.02 * np.random.default_rng(11).uniform(-1, 1, size=u.shape)
    ds_ec = ec.entropy_timederivative(u)
    ds_llf = llf.entropy_timederivative(u)
    assert ds_llf < 0
    assert abs(ds_ec) < 1e-10 * abs(ds_llf)
