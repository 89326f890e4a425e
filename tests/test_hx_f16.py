"""The FP16-split fused H*X kernel (k_hx_f16: the fused kernel's work items,
operands split into an FP16 high part and remainder scaled by a power of two
per item, one plane image read K-major by the x contraction and MN-major by
the y contraction, the next item's rows bulk-copied into shared memory).

Against the FP64 product within the mixed form's bound (2e-5 of max |Y|, as
the TF32 kernels) and against the TF32 fused kernel; blocks scaled by 1e-20
and 1e20 (the per-item scale); a smooth vector against the size of the
kinetic terms; bit for bit run to run and on two streams; a NaN reaches the
output; a block that is not 16-byte aligned and the grids the kernel declines
fall back to the other kernels."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MIXED_HX_TOL = 2e-5


@pytest.fixture(scope="module")
def torch():
    import torch as t
    assert t.cuda.is_available(), "GPU tests need a CUDA device"
    return t


def rand_block(torch, grid, nvec, seed):
    g = torch.Generator(device="cuda").manual_seed(seed)
    X = torch.randn(nvec * grid.N, dtype=torch.float64, device="cuda", generator=g)
    v = torch.randn(grid.N, dtype=torch.float64, device="cuda", generator=g)
    return X, v


def rel_err(a, b):
    return float((a - b).abs().max()) / float(b.abs().max())


@pytest.mark.parametrize("n,nvec", [(8, 3), (16, 2), (32, 40), (48, 4), (64, 4), (80, 2), (96, 8)])
def test_f16_matches_fp64_and_tf32(pg, torch, n, nvec):
    grid = pg.Grid(n, 0.615 * (n + 1))
    grid.set_hx_kernel(3)
    assert grid.hx_plan(nvec).startswith("FP16 split"), grid.hx_plan(nvec)
    X, v = rand_block(torch, grid, nvec, n + nvec)
    y64 = grid.hx(v, X, nvec=nvec, precision=pg.PG_FP64)
    y16 = grid.hx(v, X, nvec=nvec, precision=pg.PG_MIXED)
    assert rel_err(y16, y64) <= MIXED_HX_TOL
    grid.set_hx_kernel(2)
    yt = grid.hx(v, X, nvec=nvec, precision=pg.PG_MIXED)
    assert rel_err(yt, y64) <= MIXED_HX_TOL
    assert rel_err(y16, yt) <= 2 * MIXED_HX_TOL
    grid.set_hx_kernel(0)


def test_f16_is_the_automatic_choice_off_the_table(pg, torch):
    # grid sizes the tuned table does not list take the FP16-split kernel
    for n in (8, 16, 40):
        assert pg.Grid(n, 0.615 * (n + 1)).hx_plan(4).startswith("FP16 split"), n


@pytest.mark.parametrize("scale", [1e-20, 1e20])
def test_f16_scaled_blocks(pg, torch, scale):
    grid = pg.Grid(48, 30.0)
    grid.set_hx_kernel(3)
    X, v = rand_block(torch, grid, 3, 7)
    X = X * scale
    y64 = grid.hx(v, X, nvec=3, precision=pg.PG_FP64)
    y16 = grid.hx(v, X, nvec=3, precision=pg.PG_MIXED)
    assert rel_err(y16, y64) <= MIXED_HX_TOL


def test_f16_smooth_vector(pg, torch):
    # the half-box ground state on the c2 grid: the error is bounded by the
    # size of the kinetic terms, as for the TF32 kernels
    grid = pg.Grid(64, 40.0)
    grid.set_hx_kernel(3)
    w = grid.piab()
    v = torch.zeros_like(w)
    y64 = grid.hx(v, w, nvec=1, precision=pg.PG_FP64)
    y16 = grid.hx(v, w, nvec=1, precision=pg.PG_MIXED)
    scale = sum(float(np.abs(grid.kinetic(a)).sum(axis=1).max()) for a in range(3)) * float(w.abs().max())
    assert float((y16 - y64).abs().max()) / scale < 2e-6


def test_f16_repeats_and_two_streams(pg, torch):
    grid = pg.Grid(64, 40.0)
    grid.set_hx_kernel(3)
    X1, v = rand_block(torch, grid, 5, 3)
    X2, _ = rand_block(torch, grid, 5, 4)
    ref1 = grid.hx(v, X1, nvec=5, precision=pg.PG_MIXED)
    ref2 = grid.hx(v, X2, nvec=5, precision=pg.PG_MIXED)
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    torch.cuda.synchronize()
    outs = []
    for _ in range(4):
        outs.append(grid.hx(v, X1, nvec=5, precision=pg.PG_MIXED, stream=s1.cuda_stream, wait=False))
        outs.append(grid.hx(v, X2, nvec=5, precision=pg.PG_MIXED, stream=s2.cuda_stream, wait=False))
    torch.cuda.synchronize()
    grid.check()
    for k, y in enumerate(outs):
        assert torch.equal(y, ref1 if k % 2 == 0 else ref2), k


def test_f16_nan_reaches_output(pg, torch):
    grid = pg.Grid(32, 20.0)
    grid.set_hx_kernel(3)
    X, v = rand_block(torch, grid, 2, 5)
    X[grid.N + 777] = float("nan")
    y = grid.hx(v, X, nvec=2, precision=pg.PG_MIXED)
    assert torch.isnan(y[grid.N:]).any()
    assert not torch.isnan(y[:grid.N]).any()


def test_f16_unaligned_block_falls_back(pg, torch):
    grid = pg.Grid(32, 20.0)
    X, v = rand_block(torch, grid, 3, 6)
    buf = torch.empty(3 * grid.N + 1, dtype=torch.float64, device="cuda")
    buf[1:] = X
    Xu = buf[1:]  # 8 bytes past a 16-byte boundary
    y64 = grid.hx(v, X, nvec=3, precision=pg.PG_FP64)
    yu = grid.hx(v, Xu, nvec=3, precision=pg.PG_MIXED)
    assert rel_err(yu, y64) <= MIXED_HX_TOL


def test_f16_declines(pg, torch):
    # odd nx, axes with different matrices, more than 96 points
    for n, L in [((33, 33, 33), 20.0), ((32, 32, 40), 20.0), ((32, 32, 32), (20.0, 20.0, 21.0)),
                 ((112, 112, 112), 60.0)]:
        grid = pg.Grid(n, L)
        assert not grid.hx_plan().startswith("FP16 split"), (n, grid.hx_plan())
        with pytest.raises(pg.PiscesError) as e:
            grid.set_hx_kernel(3)
        assert e.value.status == pg.PG_UNSUPPORTED
