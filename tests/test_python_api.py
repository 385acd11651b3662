"""The Python wrappers of the serving and mixed-batch entry points
(sfft_gb300/serving.py) and the voted option of the binding class."""
import numpy as np
import pytest


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except ImportError:
        return False


def test_without_a_gpu_the_wrappers_refuse():
    if _has_gpu():
        pytest.skip("a CUDA device is present")
    from sfft_gb300.serving import MixedBatch, Server
    with pytest.raises(RuntimeError, match="CUDA"):
        Server()
    with pytest.raises(RuntimeError, match="CUDA"):
        MixedBatch([(1 << 16, 50, 2, "fp64")])


@pytest.mark.gpu
def test_server_and_mixed_batch_match_the_oracle(oracle_lib):
    if not _has_gpu():
        pytest.skip("no CUDA device")
    import torch
    from sfft_gb300 import build, signals
    from sfft_gb300.serving import MixedBatch, Server
    build.build()
    shapes = [(1 << 16, 50), (1 << 17, 64)]
    xs = [signals.make_signal(n, k, 70 + i)[0] for i, (n, k) in enumerate(shapes)]
    ref = [oracle_lib.OraclePlan(n, k, 1).exec(x, seed=5 + i) for i, ((n, k), x) in enumerate(zip(shapes, xs))]
    srv = Server(max_batch=4)
    ids = [srv.submit(torch.from_numpy(x).cuda(), k, version=2, precision="fp64", seed=5 + i)
           for i, ((n, k), x) in enumerate(zip(shapes, xs))]
    for i in reversed(range(len(ids))):          # any order
        gi, gv, lat = srv.wait(ids[i])
        o = np.argsort(gi, kind="stable")
        np.testing.assert_array_equal(gi[o], ref[i][0])
        np.testing.assert_array_equal(gv[o], ref[i][1])
        assert lat > 0
    srv.close()
    mb = MixedBatch([(n, k, 2, "fp64") for n, k in shapes])
    dev = [torch.from_numpy(x).cuda() for x in xs]
    for _ in range(2):                           # direct run, then a graph replay
        mb.run(dev, seeds=[5, 6])
        for i in range(len(shapes)):
            gi, gv = mb.result(i)
            o = np.argsort(gi, kind="stable")
            np.testing.assert_array_equal(gi[o], ref[i][0])
            np.testing.assert_array_equal(gv[o], ref[i][1])
    mb.close()


@pytest.mark.gpu
def test_binding_voted_option():
    if not _has_gpu():
        pytest.skip("no CUDA device")
    from sfft_gb300 import build, signals
    from sfft_gb300.sfft import sfft
    build.build()
    n, k = 1 << 18, 100
    x, pos, vals = signals.make_signal(n, k, 3)
    full = sfft(n, k, 2)
    voted = sfft(n, k, 2, voted=True)
    fi, fv = full.execute_sparse(x)
    vi, vv = voted.execute_sparse(x)
    assert vi.size < fi.size // 10
    est = np.zeros(n, dtype=complex)
    est[vi] = np.conj(vv)
    assert np.max(np.abs(est[pos] - vals)) < 1e-6
    with pytest.raises(ValueError):
        sfft(1 << 16, 50, 1, voted=True)
