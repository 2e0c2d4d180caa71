"""Device graph generators against the oracle's CPU generators, and MSF
parity on their graphs.

The device generators must be bit-identical to the oracle's (same seeded
definition), so that GPU and CPU runs of a workload see the same input.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev_rgg(kamsta, ctx, n, radius, seed, wmax=254):
    import torch
    md = ctx.gen_rgg2d_dev(n, radius, seed, wmax)  # count only
    d = torch.empty((max(md, 1), 3), dtype=torch.int32, device="cuda")
    got = ctx.gen_rgg2d_dev(n, radius, seed, wmax, d.data_ptr(), md)
    assert got == md
    torch.cuda.synchronize()
    return d[:md].cpu().numpy().view(np.uint32).reshape(-1).view(kamsta.WEDGE)


@pytest.mark.parametrize("n,deg,seed", [(1, 4.0, 1), (2, 4.0, 1), (100, 4.0, 2), (1000, 16.0, 3),
                                        (1 << 16, 16.0, 4), (1 << 18, 8.0, 5),
                                        (1 << 20, 16.0, 6)])
def test_rgg2d_matches_oracle(kamsta, oracle, n, deg, seed):
    ctx = kamsta.Context(0)
    r = oracle.rgg_radius(n, deg)
    assert np.array_equal(_dev_rgg(kamsta, ctx, n, r, seed), oracle.gen_rgg2d(n, r, seed))


@pytest.mark.parametrize("radius", [0.0, 1.0, 0.3])
def test_rgg2d_extreme_radii(kamsta, oracle, radius):
    ctx = kamsta.Context(0)
    assert np.array_equal(_dev_rgg(kamsta, ctx, 300, radius, 9), oracle.gen_rgg2d(300, radius, 9))


def test_rgg2d_capacity_error(kamsta):
    import torch
    ctx = kamsta.Context(0)
    n = 5000
    r = 0.02
    md = ctx.gen_rgg2d_dev(n, r, 1, 254)
    assert md > 10
    d = torch.empty((md, 3), dtype=torch.int32, device="cuda")
    with pytest.raises(kamsta.KamstaError):
        ctx.gen_rgg2d_dev(n, r, 1, 254, d.data_ptr(), md - 1)


@pytest.mark.parametrize("algo", ["boruvka_plain", "boruvka_local", "filter_boruvka"])
@pytest.mark.parametrize("n,deg", [(1 << 12, 4.0), (1 << 16, 16.0), (1 << 18, 6.0)])
def test_mst_on_rgg2d(kamsta, oracle, algo, n, deg):
    from tests.test_parity_gpu import _check, _configs
    fn, cfg = _configs(kamsta)[algo]
    e = oracle.gen_rgg2d(n, oracle.rgg_radius(n, deg), 40 + n % 7)
    _check(oracle, fn(e, cfg, n=n), e, n)


def _dev_rhg(kamsta, ctx, n, gamma, k, seed, wmax=254):
    import torch
    md = ctx.gen_rhg_dev(n, gamma, k, seed, wmax)
    d = torch.empty((max(md, 1), 3), dtype=torch.int32, device="cuda")
    assert ctx.gen_rhg_dev(n, gamma, k, seed, wmax, d.data_ptr(), md) == md
    torch.cuda.synchronize()
    return d[:md].cpu().numpy().view(np.uint32).reshape(-1).view(kamsta.WEDGE)


@pytest.mark.parametrize("n,gamma,k,seed", [(1, 3.0, 16, 1), (2, 3.0, 4, 2), (300, 3.0, 16, 3),
                                            (5000, 2.5, 10, 4), (1 << 16, 3.0, 16, 5),
                                            (1 << 18, 3.0, 16, 6), (1 << 17, 4.0, 8, 7)])
def test_rhg_matches_oracle(kamsta, oracle, n, gamma, k, seed):
    ctx = kamsta.Context(0)
    assert np.array_equal(_dev_rhg(kamsta, ctx, n, gamma, k, seed),
                          oracle.gen_rhg(n, gamma, k, seed))


@pytest.mark.parametrize("algo", ["boruvka_plain", "boruvka_local", "filter_boruvka",
                                  "filter_dedupe"])
@pytest.mark.parametrize("n,k", [(1 << 12, 8.0), (1 << 16, 16.0), (1 << 19, 16.0)])
def test_mst_on_rhg(kamsta, oracle, algo, n, k):
    from tests.test_parity_gpu import _check, _configs
    fn, cfg = _configs(kamsta)[algo]
    e = oracle.gen_rhg(n, 3.0, k, 50 + n % 11)
    _check(oracle, fn(e, cfg, n=n), e, n)


@pytest.mark.parametrize("family", ["rgg2d", "rhg"])
def test_filter_boruvka_geometric_config_exactness(kamsta, oracle, family):
    """The geometric / skewed configuration (filter-Boruvka on RGG-2D and RHG
    with average degree 16) at n=2^21, checked against Kruskal."""
    n = 1 << 21
    e = (oracle.gen_rgg2d(n, oracle.rgg_radius(n, 16), 2024) if family == "rgg2d"
         else oracle.gen_rhg(n, 3.0, 16, 2024))
    from tests.test_parity_gpu import _check
    _check(oracle, kamsta.filter_boruvka(e, kamsta.AlgorithmConfig(), n=n), e, n)


def _dev_counted(kamsta, gen, *args):
    """Count, allocate, write: the counting convention of the generators."""
    import torch
    md = gen(*args)
    d = torch.empty((max(md, 1), 3), dtype=torch.int32, device="cuda")
    assert gen(*args, d_out=d.data_ptr(), capacity=md) == md
    torch.cuda.synchronize()
    return d[:md].cpu().numpy().view(np.uint32).reshape(-1).view(kamsta.WEDGE)


@pytest.mark.parametrize("X,Y,Z,p,periodic", [(1, 1, 1, 1.0, True), (2, 2, 2, 1.0, True),
                                              (5, 3, 1, 1.0, False), (7, 1, 1, 1.0, True),
                                              (1024, 1024, 1, 1.0, True),
                                              (64, 64, 64, 1.0, True), (300, 200, 1, 0.7, False),
                                              (40, 50, 60, 0.45, True)])
def test_grid_matches_oracle(kamsta, oracle, X, Y, Z, p, periodic):
    ctx = kamsta.Context(0)
    got = _dev_counted(kamsta, lambda **kw: ctx.gen_grid_dev(X, Y, Z, p, periodic, 21, 254, **kw))
    assert np.array_equal(got, oracle.gen_grid(X, Y, Z, p, periodic, 21))


@pytest.mark.parametrize("n,deg,seed", [(1, 8.0, 1), (2, 8.0, 2), (300, 8.0, 3),
                                        (1 << 16, 16.0, 4), (1 << 18, 10.0, 5)])
def test_rgg3d_matches_oracle(kamsta, oracle, n, deg, seed):
    ctx = kamsta.Context(0)
    r = oracle.rgg3d_radius(n, deg)
    got = _dev_counted(kamsta, lambda **kw: ctx.gen_rgg3d_dev(n, r, seed, 254, **kw))
    assert np.array_equal(got, oracle.gen_rgg3d(n, r, seed))


@pytest.mark.parametrize("L,samples,seed,abc", [(1, 10, 1, (0.57, 0.19, 0.19)),
                                                (10, 3000, 3, (0.57, 0.19, 0.19)),
                                                (16, 1 << 20, 4, (0.57, 0.19, 0.19)),
                                                (20, 1 << 22, 5, (0.45, 0.15, 0.15)),
                                                (12, 1 << 16, 6, (0.25, 0.25, 0.25))])
def test_rmat_matches_oracle(kamsta, oracle, L, samples, seed, abc):
    ctx = kamsta.Context(0)
    got = _dev_counted(kamsta, lambda **kw: ctx.gen_rmat_dev(L, samples, seed, *abc, 254, **kw))
    assert np.array_equal(got, oracle.gen_rmat(L, samples, seed, *abc))


def test_generator_capacity_errors(kamsta):
    import torch
    ctx = kamsta.Context(0)
    for gen in (lambda **kw: ctx.gen_grid_dev(30, 30, 1, **kw),
                lambda **kw: ctx.gen_rgg3d_dev(4000, 0.1, 1, **kw),
                lambda **kw: ctx.gen_rmat_dev(12, 1 << 14, 1, **kw)):
        md = gen()
        assert md > 10
        d = torch.empty((md, 3), dtype=torch.int32, device="cuda")
        with pytest.raises(kamsta.KamstaError):
            gen(d_out=d.data_ptr(), capacity=md - 1)
    with pytest.raises(kamsta.KamstaError):
        ctx.gen_rmat_dev(32, 10, 1)
    with pytest.raises(kamsta.KamstaError):
        ctx.gen_rmat_dev(10, 10, 1, 0.6, 0.3, 0.2)
    with pytest.raises(kamsta.KamstaError):
        ctx.gen_grid_dev(1 << 16, 1 << 16, 1)


@pytest.mark.parametrize("algo", ["boruvka_plain", "boruvka_local", "filter_boruvka",
                                  "filter_dedupe"])
@pytest.mark.parametrize("family", ["grid2d", "grid3d", "rgg3d", "rmat"])
def test_mst_on_more_families(kamsta, oracle, algo, family):
    """MSF parity on lattices (many equal-weight ties, long paths), 3-D
    geometric graphs and R-MAT (hubs at the smallest ids, isolated
    vertices)."""
    from tests.test_parity_gpu import _check, _configs
    fn, cfg = _configs(kamsta)[algo]
    if family == "grid2d":
        n, e = 300 * 200, oracle.gen_grid(300, 200, 1, 0.8, True, 3, 8)
    elif family == "grid3d":
        n, e = 40 * 40 * 40, oracle.gen_grid(40, 40, 40, 1.0, False, 4, 4)
    elif family == "rgg3d":
        n = 1 << 17
        e = oracle.gen_rgg3d(n, oracle.rgg3d_radius(n, 12), 5)
    else:
        n, e = 1 << 18, oracle.gen_rmat(18, 1 << 22, 6)
    _check(oracle, fn(e, cfg, n=n), e, n)


@pytest.mark.parametrize("mode", [1, 2])
@pytest.mark.parametrize("dim", [2, 3])
def test_distance_weights_match_oracle(kamsta, oracle, mode, dim):
    """Euclidean / squared-Euclidean weights of the geometric generators are
    bit-identical to the oracle's (exact integer rules)."""
    ctx = kamsta.Context(0)
    n = 1 << 16
    if dim == 2:
        r = oracle.rgg_radius(n, 12)
        got = _dev_counted(kamsta, lambda **kw: ctx.gen_rgg2d_dev(n, r, 11, 254, distance=mode,
                                                                 **kw))
        ref = oracle.gen_rgg2d(n, r, 11, 254, distance=mode)
    else:
        r = oracle.rgg3d_radius(n, 12)
        got = _dev_counted(kamsta, lambda **kw: ctx.gen_rgg3d_dev(n, r, 11, 254, distance=mode,
                                                                 **kw))
        ref = oracle.gen_rgg3d(n, r, 11, 254, distance=mode)
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("algo", ["boruvka_plain", "boruvka_local", "filter_boruvka"])
def test_mst_on_euclidean_rgg(kamsta, oracle, algo):
    """Distance weights make the MSF geometric (and tie often: 254 levels)."""
    from tests.test_parity_gpu import _check, _configs
    fn, cfg = _configs(kamsta)[algo]
    n = 1 << 17
    e = oracle.gen_rgg2d(n, oracle.rgg_radius(n, 10), 12, 254, distance=1)
    _check(oracle, fn(e, cfg, n=n), e, n)
