"""The measurement probes behind the bench's roofline figures: sequential read bandwidth of a
buffer (L2-resident or in HBM) and the rate of random 32-byte reads, the access a density-cell
lookup makes."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(built):
    import narvalengine_gb300 as ne
    c = ne.Context(0)
    yield c
    c.close()


def test_read_bandwidth_l2_above_hbm(ctx):
    l2 = ctx.read_bandwidth(48 << 20, 5)
    hbm = ctx.read_bandwidth(2 << 30, 3)
    assert 1000 < hbm < 12000, hbm
    assert l2 > 1.3 * hbm, (l2, hbm)


def test_random_read_rate(ctx):
    import narvalengine_gb300 as ne
    in_l2 = ctx.random_read_rate(32 << 20, 3)
    in_hbm = ctx.random_read_rate(2 << 30, 3)
    # 32 bytes per read: below the sequential rates, and the L2-resident buffer serves more
    assert 1e9 < in_hbm < 12000e9 / 32, in_hbm
    assert in_l2 > in_hbm, (in_l2, in_hbm)
    with pytest.raises(ne.NarvalError):
        ctx.random_read_rate(16, 1)
    with pytest.raises(ne.NarvalError):
        ctx.random_read_rate(1 << 20, 0)
