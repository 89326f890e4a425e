"""pg_block_gram_noalloc: the Gram product with its reduction scratch in a
fixed device array instead of allocated memory.  Compared, bit for bit,
with pg_block_gram on two calls in a row of different shapes (the second
call reuses the scratch the first one wrote); around each call the
library's device-allocation count and the device's free memory stay the
same; sizes beyond the fixed scratch are refused.  Collected last, and
self-contained, so it passes alone and after the other tests."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch as t
    assert t.cuda.is_available(), "GPU tests need a CUDA device"
    return t


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_noalloc_gram_matches_block_gram_twice(pg, torch, precision):
    g = torch.Generator(device="cuda").manual_seed(21)
    n = 64 ** 3
    cases = [(40, 4), (9, 9)]  # 160 and 81 outputs: both within the 256-output scratch
    for na, nb in cases:
        P = torch.randn(na, n, dtype=torch.float64, device="cuda", generator=g)
        Q = torch.randn(nb, n, dtype=torch.float64, device="cuda", generator=g)
        ref = pg.block_gram(P, Q, precision=precision)
        out = torch.full((na * nb,), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        allocs0 = pg.lib().pg_device_allocations()
        free0 = torch.cuda.mem_get_info()[0]
        got = pg.block_gram_noalloc(P, Q, out, precision=precision)
        torch.cuda.synchronize()
        assert pg.lib().pg_device_allocations() == allocs0, (na, nb)
        assert torch.cuda.mem_get_info()[0] == free0, (na, nb)
        assert torch.equal(got, ref), (na, nb)


def test_noalloc_gram_refuses_more_than_its_scratch(pg, torch):
    P = torch.zeros(17, 1000, dtype=torch.float64, device="cuda")
    Q = torch.zeros(16, 1000, dtype=torch.float64, device="cuda")  # 272 outputs > 256
    out = torch.empty(17 * 16, dtype=torch.float64, device="cuda")
    with pytest.raises(pg.PiscesError) as e:
        pg.block_gram_noalloc(P, Q, out)
    assert e.value.status == pg.PG_BAD_ARG and "256" in str(e.value)
