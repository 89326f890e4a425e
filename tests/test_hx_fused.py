"""The fused mixed-form H*X kernel (k_hx_fused: x and y contractions of each
grid plane in one tensor-memory tile, z contraction of 128-line tiles, one
persistent launch with a work queue and per-vector completion counters).

Against the FP64 product within the mixed form's bound (2e-5 of max |Y|,
as the three-pass kernels), against the three-pass kernels, bit for bit run
to run, with several launches in a row and on two streams at once (each
stream has its own counters), and the grids it declines."""
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


@pytest.mark.parametrize("n,nvec", [((8, 8, 8), 3), ((33, 33, 33), 5), ((48, 48, 48), 4), ((64, 64, 64), 4),
                                    ((80, 80, 80), 2), ((96, 96, 96), 8), ((24, 20, 28), 7), ((3, 5, 7), 2),
                                    ((2, 17, 9), 3), ((32, 32, 32), 40)])
def test_fused_matches_fp64_and_three_pass(pg, torch, n, nvec):
    grid = pg.Grid(n, tuple(0.6 * (k + 1) for k in n))
    grid.set_hx_kernel(2)
    assert grid.hx_plan().startswith("fused"), grid.hx_plan()
    X, v = rand_block(torch, grid, nvec, sum(n) + nvec)
    y64 = grid.hx(v, X, nvec=nvec, precision=pg.PG_FP64)
    yf = grid.hx(v, X, nvec=nvec, precision=pg.PG_MIXED)
    assert rel_err(yf, y64) <= MIXED_HX_TOL
    grid.set_hx_kernel(1)
    assert grid.hx_plan().startswith("three axis passes")
    y3 = grid.hx(v, X, nvec=nvec, precision=pg.PG_MIXED)
    assert rel_err(y3, y64) <= MIXED_HX_TOL
    assert rel_err(yf, y3) <= 2 * MIXED_HX_TOL
    grid.set_hx_kernel(0)


def test_fused_repeats_bit_for_bit(pg, torch):
    # several launches in a row on one stream reuse its counter block, which
    # the last CTA of each launch resets; the output is the same bits
    grid = pg.Grid((64, 64, 64), (40.0, 40.0, 40.0))
    grid.set_hx_kernel(2)
    X, v = rand_block(torch, grid, 6, 3)
    first = grid.hx(v, X, nvec=6, precision=pg.PG_MIXED)
    for _ in range(5):
        Y = grid.hx(v, X, nvec=6, precision=pg.PG_MIXED, wait=False)
    grid.check()
    assert torch.equal(Y, first)


def test_fused_two_streams_at_once(pg, torch):
    # the same grid on two streams concurrently: separate counter blocks
    grid = pg.Grid((48, 48, 48), (30.0, 30.0, 30.0))
    grid.set_hx_kernel(2)
    X1, v = rand_block(torch, grid, 5, 8)
    X2, _ = rand_block(torch, grid, 5, 9)
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


def test_fused_smooth_vector(pg, torch):
    # a smooth vector (the half-box ground state) on the c2 grid: its kinetic
    # sums cancel strongly, so the error is bounded by the size of the terms
    # (sum over axes of the largest row sum of |T| times max |x|), as for the
    # three-pass kernels, and is no larger than theirs
    n, L = (64, 64, 64), (40.0, 40.0, 40.0)
    grid = pg.Grid(n, L)
    grid.set_hx_kernel(2)
    w = grid.piab()
    v = torch.zeros_like(w)
    y64 = grid.hx(v, w, nvec=1, precision=pg.PG_FP64)
    yf = grid.hx(v, w, nvec=1, precision=pg.PG_MIXED)
    scale = sum(float(np.abs(grid.kinetic(a)).sum(axis=1).max()) for a in range(3)) * float(w.abs().max())
    err_f = float((yf - y64).abs().max())
    assert err_f / scale < 2e-6
    grid.set_hx_kernel(1)
    err_3 = float((grid.hx(v, w, nvec=1, precision=pg.PG_MIXED) - y64).abs().max())
    assert err_f <= 2 * err_3 + 1e-9 * scale, (err_f, err_3)


def test_fused_declines_large_axes(pg, torch):
    # more than 112 points on an axis (K chunks) or 128 along x: three passes
    for n in [(160, 24, 20), (24, 24, 136), (129, 2, 3)]:
        grid = pg.Grid(n, tuple(0.6 * (k + 1) for k in n))
        assert grid.hx_plan().startswith("three axis passes"), (n, grid.hx_plan())
        with pytest.raises(pg.PiscesError) as e:
            grid.set_hx_kernel(2)
        assert e.value.status == pg.PG_UNSUPPORTED
    with pytest.raises(pg.PiscesError) as e:
        pg.Grid((8, 8, 8), (5.0, 5.0, 5.0)).set_hx_kernel(4)
    assert e.value.status == pg.PG_BAD_ARG
