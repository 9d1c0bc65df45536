"""The mixed path's state conversions: an FP64 state uploaded into a mixed
context becomes float-float pairs hi = fl32(x), lo = fl32(x - hi) (both rounded
to nearest even), and a download returns hi + lo in FP64.  The kernels do this
with integer operations on the bit patterns where the exponents allow and
with the conversion instructions elsewhere; both must give the IEEE results
bit for bit, over the whole double range, ties, signed zeros, subnormals,
infinities and NaN included, through every upload path (pageable and
page-locked host memory, the prefetch slots; the 2D shock-capturing context's
conversion that also writes rho*p).  That conversion also makes the CFL
reduction of the new state, which must give the separate reduction's step
size exactly."""
import numpy as np
import pytest

from _gpu_cases import build

pytestmark = pytest.mark.gpu

KHI = dict(ndims=2, polydeg=3, level=4, xmin=[-1.0, -1.0], xmax=[1.0, 1.0], vi="hg",
           volume_flux="ranocha", surface_flux="llf", ic="kelvin_helmholtz",
           alpha_max=0.002, alpha_min=0.0001)
MMS3 = dict(ndims=3, polydeg=3, level=2, xmin=[0.0] * 3, xmax=[2.0] * 3, vi="fluxdiff",
            volume_flux="ranocha", surface_flux="llf", ic="convergence_test",
            source="convergence_test")


def _tricky_values(n, seed):
    rng = np.random.default_rng(seed)
    with np.errstate(over="ignore"):  # the largest exponents give infinities
        x = np.ldexp(rng.uniform(-1.0, 1.0, n), rng.integers(-1100, 1030, n))
    k = n // 4  # ties and near-ties of the rounding to 24 bits
    t = rng.integers(1 << 24, 1 << 25, k).astype(np.float64) + rng.choice([0.5, 0.25, 0.75], k)
    x[:k] = np.ldexp(t, rng.integers(-80, 100, k)) * rng.choice([-1.0, 1.0], k)
    k2 = n // 4  # the exponent window of the integer path and just outside it
    x[k:k + k2] = np.ldexp(rng.uniform(0.5, 1.0, k2), rng.integers(-78, 130, k2)) * rng.choice([-1.0, 1.0], k2)
    special = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, -5e-324, 1e-310, 1e-40, -3e-39,
                        np.finfo(np.float32).max, np.nextafter(np.float64(np.finfo(np.float32).max), np.inf),
                        1e300, -1e300, 1.0, np.nextafter(1.0, 2.0), np.nextafter(1.0, 0.0),
                        2.0 ** -74, 2.0 ** -75, 2.0 ** 126, 2.0 ** 127, 1.0 + 2.0 ** -24])
    x[k + k2:k + k2 + special.size] = special
    return x


def _expected_roundtrip(x):
    with np.errstate(over="ignore", invalid="ignore"):
        hi = x.astype(np.float32)
        lo = (x - hi.astype(np.float64)).astype(np.float32)
        return hi.astype(np.float64) + lo.astype(np.float64)


def _check(got, x):
    want = _expected_roundtrip(x)
    same = (got.view(np.uint64) == want.view(np.uint64)) | (np.isnan(got) & np.isnan(want))
    if not same.all():
        i = np.nonzero(~same)[0][0]
        raise AssertionError(f"{(~same).sum()} values differ; first: x={x[i].hex()} "
                             f"got={got[i].hex()} want={want[i].hex()}")


@pytest.mark.parametrize("case", [KHI, MMS3], ids=["khi2d_rho_p", "mms3d"])
def test_upload_download_bitwise(case):
    torch = pytest.importorskip("torch")
    semi, _ = build(case, precision="mixed")
    ctx = semi.device_context
    for seed in (1, 2):
        x = _tricky_values(semi.nvalues, seed)
        ctx.upload(x.reshape(semi.u_shape))  # pageable: staged, converted on the device
        _check(ctx.download().reshape(-1), x)
        pinned = torch.from_numpy(x.copy()).pin_memory()
        ctx.upload(pinned.numpy().reshape(semi.u_shape))  # page-locked: read in place
        out = torch.empty_like(pinned).pin_memory()
        ctx.download(out.numpy().reshape(semi.u_shape))
        _check(out.numpy(), x)
        ctx.prefetch(seed % 2, pinned.data_ptr())  # the prefetch slots
        ctx.load_prefetched(seed % 2)
        ctx.fetch(seed % 2, out.data_ptr())
        ctx.transfer_wait(seed % 2, 1)
        _check(out.numpy(), x)
        # page-locked buffers 8 bytes off a 16-byte boundary (the 8-byte kernels)
        off = torch.zeros(x.size + 1, dtype=torch.float64).pin_memory()
        off[1:] = torch.from_numpy(x)
        ctx.upload(off.numpy()[1:].reshape(semi.u_shape))
        off.zero_()
        ctx.download(off.numpy()[1:].reshape(semi.u_shape))
        _check(off.numpy()[1:], x)
    ctx.transfer_join()
    ctx.synchronize()


BLAST_REFINED = dict(ndims=2, polydeg=3, level=4, xmin=[-1.5, -1.5], xmax=[1.5, 1.5], vi="hg",
                     volume_flux="ranocha", surface_flux="llf", ic="gaussian_blast",
                     ic_params=[1e-5, 1.0, 0.25], alpha_max=0.5, alpha_min=0.001,
                     refinement_patches=(dict(type="box", coordinates_min=(-0.5, -0.5),
                                              coordinates_max=(0.5, 0.5)),))
KHI_WALLS = dict(KHI, boundary="slip_wall")


@pytest.mark.parametrize("case", [KHI, BLAST_REFINED, KHI_WALLS], ids=["khi", "blast_refined", "khi_walls"])
def test_upload_cfl_reduction_matches_separate_reduction(case):
    # an upload into a 2D shock-capturing mixed context reduces the CFL speed
    # of the new state in its conversion pass; the first step size must equal
    # the one from the separate reduction (forced here by handing out the state
    # pointer, after which the state counts as changed)
    semi, _ = build(case, precision="mixed")
    ctx = semi.device_context
    u0 = semi.compute_coefficients(0.0)
    ctx.upload(u0)
    ctx.step(3, 1.0, 10.0, 0.0)
    u = ctx.download()
    torch = pytest.importorskip("torch")
    off = torch.zeros(u.size + 1, dtype=torch.float64).pin_memory()
    off[1:] = torch.from_numpy(u.reshape(-1))
    u_off = off.numpy()[1:].reshape(semi.u_shape)  # 8 bytes off a 16-byte boundary
    for cfl in (1.0, 0.37):
        ctx.upload(u)
        t_fused, _ = ctx.step(1, cfl, 10.0, 0.0)
        ctx.upload(u_off)
        t_fused8, _ = ctx.step(1, cfl, 10.0, 0.0)
        ctx.upload(u)
        ctx.state_ptr()
        t_sep, _ = ctx.step(1, cfl, 10.0, 0.0)
        assert t_fused == t_sep and t_fused8 == t_sep and t_fused > 0
        ctx.upload(u)
        assert ctx.max_dt() * cfl == pytest.approx(t_fused, rel=1e-12)
