"""AMR on the host (CPU only): the TreeMesh adaptation (refine! with 2:1
rebalancing, then coarsen! with its balance rule; amr.jl:244-392,
abstract_tree.jl:317-618) and the transfer map it hands to the device must
reproduce the oracle's restatement: the same elements, containers and --
applied with the L2 adaptor matrices -- the same transferred state."""
import numpy as np
import pytest

import trixi_gb300 as T
from oracle import oracle as O


def transfer(u_old, src, kind, mortar, ndims):
    """The projection tg_adapt_state performs, in numpy (test reference)."""
    n = u_old.shape[1]
    F = (mortar.forward_lower, mortar.forward_upper)
    R = (mortar.reverse_lower, mortar.reverse_upper)
    out = np.zeros((len(src),) + u_old.shape[1:])
    for e, (s0, k) in enumerate(zip(src, kind)):
        if k == 0:
            out[e] = u_old[s0]
            continue
        parts = [(s0, k - 1, F)] if k > 0 else [(s0 + q, q, R) for q in range(1 << ndims)]
        for se, q, M in parts:
            if ndims == 2:  # arrays are [j, i, v]
                out[e] += np.einsum("ik,jl,lkv->jiv", M[q & 1], M[(q >> 1) & 1], u_old[se])
            else:  # [k, j, i, v]
                out[e] += np.einsum("ia,jb,kc,cbav->kjiv", M[q & 1], M[(q >> 1) & 1],
                                    M[(q >> 2) & 1], u_old[se])
    return out


def _semi(ndims, level, lo, hi, ic, patches=()):
    mesh = T.TreeMesh([lo] * ndims, [hi] * ndims, initial_refinement_level=level,
                      refinement_patches=patches)
    eq = T.CompressibleEulerEquations2D(1.4) if ndims == 2 else T.CompressibleEulerEquations3D(1.4)
    return T.SemidiscretizationHyperbolic(mesh, eq, ic, T.DGSEM(polydeg=3))


def _check_same_mesh(semi, orc):
    om = orc.mesh()
    assert semi.nelements == orc.nelements
    np.testing.assert_array_equal(semi.mesh.element_levels(), orc.element_levels())
    np.testing.assert_array_equal(semi.neighbor_ids, om["neighbor_ids"])
    ids, ls, orient = orc.mortars()
    np.testing.assert_array_equal(semi.mortar_neighbor_ids, ids)
    np.testing.assert_array_equal(semi.mortar_large_sides, ls)
    np.testing.assert_array_equal(semi.mortar_orientations, orient)
    np.testing.assert_allclose(semi.node_coordinates, om["node_coordinates"], rtol=0, atol=1e-13)


@pytest.mark.parametrize("ndims,level", [(2, 4), (3, 2)])
def test_random_adaptation_matches_oracle(ndims, level):
    rng = np.random.default_rng(17 + ndims)
    semi = _semi(ndims, level, -1.0, 1.0, T.initial_condition_weak_blast_wave)
    orc = O.Oracle(ndims, 3, level, [-1.0] * ndims, [1.0] * ndims)
    u = semi.compute_coefficients(0.0)
    u = u * (1 + 0.01 * rng.uniform(-1, 1, u.shape))
    passes = 0
    kinds = set()
    for step in range(6):
        lam = rng.choice([-1, 0, 1], size=semi.nelements, p=[0.5, 0.3, 0.2]).astype(np.int8)
        if step % 3 == 2:
            lam[:] = -1  # everything wants to coarsen: only balanced parents may
        changed, src, kind = semi.mesh.adapt(lam)
        ochanged, u_orc = orc.adapt_with(u, lam)
        assert changed == ochanged
        if not changed:
            continue
        passes += 1
        semi._setup_containers()
        _check_same_mesh(semi, orc)
        u_new = transfer(u, src, kind, semi.solver.mortar, ndims)
        np.testing.assert_allclose(u_new, u_orc, rtol=0, atol=1e-13 * np.abs(u_orc).max())
        assert set(np.unique(kind)) <= set(range(-1, (1 << ndims) + 1))
        kinds |= set(np.unique(kind).tolist())
        u = u_new
    assert passes >= 4
    assert -1 in kinds and 1 in kinds  # both coarsening and refinement happened


def test_only_refine_and_only_coarsen():
    semi = _semi(2, 3, -1.0, 1.0, T.initial_condition_weak_blast_wave)
    lam = np.zeros(semi.nelements, dtype=np.int8)
    lam[:4] = -1  # the four children of the first level-2 cell
    lam[-1] = 1
    changed, src, kind = semi.mesh.adapt(lam, only_coarsen=True)
    assert changed and semi.mesh.nelements == 61 and kind[0] == -1 and src[0] == 0
    lam = np.zeros(semi.mesh.nelements, dtype=np.int8)
    lam[0] = -1
    lam[-1] = 1
    changed, src, kind = semi.mesh.adapt(lam, only_refine=True)
    assert changed and semi.mesh.nelements == 64 and list(kind[-4:]) == [1, 2, 3, 4]
    changed, _, _ = semi.mesh.adapt(np.zeros(semi.mesh.nelements, dtype=np.int8))
    assert not changed


def test_controller_three_level_matches_oracle():
    # ControllerThreeLevel on the HG indicator (the blast_wave_amr settings) vs the
    # oracle's controller; indicator values come from the oracle here
    semi = _semi(2, 5, -2.0, 2.0, T.initial_condition_blast_wave)
    orc = O.Oracle(2, 3, 5, [-2.0] * 2, [2.0] * 2)
    orc.set_amr(alpha_max=0.5, alpha_min=0.001, alpha_smooth=True, base_level=4,
                med_level=5, med_threshold=0.0005, max_level=6, max_threshold=0.01)
    u = semi.compute_coefficients(0.0)
    ind = T.IndicatorHennemannGassner(semi, alpha_max=0.5, alpha_min=0.001, alpha_smooth=True,
                                      variable=T.density_pressure)
    ctrl = T.ControllerThreeLevel(semi, ind, base_level=4, med_level=5, med_threshold=0.0005,
                                  max_level=6, max_threshold=0.01)
    orc2 = O.Oracle(2, 3, 5, [-2.0] * 2, [2.0] * 2, volume_integral=O.VI_SHOCKCAPTURING_HG,
                    alpha_max=0.5, alpha_min=0.001, alpha_smooth=True)
    ctrl.indicator_values = lambda s: orc2.alpha(u)
    lam = ctrl(semi)
    np.testing.assert_array_equal(lam, orc.amr_lambda(u))
    assert set(np.unique(lam)) == {-1, 1}


def test_native_tree_rejects_invalid_input():
    from trixi_gb300 import _lib
    lib = _lib.load()
    import ctypes
    h = ctypes.c_void_p()
    lo = (ctypes.c_double * 3)(0, 0, 0)
    hi = (ctypes.c_double * 3)(1, 1, 1)
    assert lib.tg_tree_create(4, 2, lo, hi, None, ctypes.byref(h)) == _lib.TG_ERR_INVALID_ARGUMENT
    assert "ndims" in _lib.last_error()
    assert lib.tg_tree_create(2, 2, hi, lo, None, ctypes.byref(h)) == _lib.TG_ERR_INVALID_ARGUMENT
    assert lib.tg_tree_create(2, 2, lo, hi, None, ctypes.byref(h)) == _lib.TG_OK
    assert lib.tg_tree_refine_patch(h, 7, lo, hi, 0.0) == _lib.TG_ERR_INVALID_ARGUMENT
    n = ctypes.c_int64()
    assert lib.tg_tree_nelements(h, ctypes.byref(n)) == _lib.TG_OK and n.value == 16
    # no transfer map before an adaptation changed the mesh
    src = (ctypes.c_int64 * 16)()
    kind = (ctypes.c_int8 * 16)()
    assert lib.tg_tree_transfer_map(h, src, kind) == _lib.TG_ERR_INVALID_ARGUMENT
    lib.tg_tree_destroy(h)


def test_refinement_stops_at_the_maximum_level():
    # sphere patches shrinking with the cell size refine the cells around one
    # point level by level (2:1 balanced); the tree stops at level 15, and the
    # mesh constructor raises beyond it
    def patches(levels):
        return [dict(type="sphere", center=(0.01, 0.02), radius=0.75 * 2.0 / 2 ** k) for k in levels]
    mesh = T.TreeMesh((-1.0, -1.0), (1.0, 1.0), initial_refinement_level=2,
                      refinement_patches=patches(range(2, 15)))
    assert mesh.element_levels().max() == 15 and mesh.nelements < 2000
    with pytest.raises(T.TrixiGB300Error):
        T.TreeMesh((-1.0, -1.0), (1.0, 1.0), initial_refinement_level=2,
                   refinement_patches=patches(range(2, 16)))
