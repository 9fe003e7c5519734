"""Host-side pieces of bench.py that need no GPU: the algorithmic-byte
formulas the roofline uses, the --panels option and the traffic ratios."""
import bench


def test_eval_bytes_formula():
    # A and A^T once each (value + 4-byte id per nonzero), row offsets, the
    # input vector of each pass, labels (FP64), r written then read, g (FP64)
    m, n, nnz = 10, 7, 40
    p1, p2 = bench.eval_bytes(m, n, nnz, 2, 4)
    assert p1 == nnz * 6 + (m + 1) * 4 + n * 4 + m * 8 + m * 4
    assert p2 == nnz * 6 + (n + 1) * 4 + m * 4 + n * 8


class _FakeMatrix:
    def __init__(self):
        self.calls = []

    def set_panels(self, rows=-1, min_per_panel=0.0):
        self.calls.append((rows, min_per_panel))


def test_panels_option():
    A = _FakeMatrix()
    bench.set_panels(A, "auto")
    assert A.calls == []
    bench.set_panels(A, "off")
    bench.set_panels(A, "8192")
    bench.set_panels(A, "4096:1.5")
    assert A.calls == [(0, 0.0), (8192, 0.0), (4096, 1.5)]


def test_traffic_ratios():
    for storage, r in bench.NCU_TRAFFIC_RATIO.items():
        for k in ("pass1", "pass2"):
            assert 0.5 < r[k] <= 1.2, (storage, k)
        assert storage in bench.TRAFFIC_SOURCE


def test_split_arm_bytes():
    # split storage: a 4-byte FP32 value, a 2-byte residual and a 4-byte id
    # per nonzero; vectors as FP32 pairs
    m, n, nnz = 10, 7, 40
    p1, p2 = bench.train_bytes_per_eval(m, n, nnz, "split")
    assert (p1, p2) == bench.eval_bytes(m, n, nnz, 6, 8)
    assert bench.train_bytes_per_eval(m, n, nnz, "bf16") == bench.eval_bytes(m, n, nnz, 2, 4)


def test_parity_of():
    import numpy as np
    ref = {"loss": 100.0, "w": np.array([1.0, -2.0]), "trace": np.array([[1.0, 1.0, 0, 0], [1.0, 2.0, 0, 0]])}
    ok = bench.parity_of({"loss": 100.00005, "w": np.array([1.0, -2.00001]), "trace": ref["trace"]}, ref)
    assert ok["within_bar"] and ok["trials_same"]
    bad = bench.parity_of({"loss": 100.001, "w": np.array([1.0, -2.0])}, ref)
    assert not bad["within_bar"] and "trials_same" not in bad


def _replica(rank, port, out):
    import os
    os.environ.update({"WORLD_SIZE": "2", "RANK": str(rank), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import bench as b
    world, r, local = b.dist_setup(None)
    b.barrier(world)
    # each replica's step time; the job's time is the slowest replica's
    t = b.allmax(world, 10.0 + rank)
    out.put((r, world, local, t))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_replicas_gloo_two_ranks():
    # the bench's N > 1 path: replicas (nothing sharded), a barrier and the
    # max over ranks of the timed region, here on two gloo ranks on the CPU
    import multiprocessing as mp
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    ps = [ctx.Process(target=_replica, args=(r, port, out)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(out.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == [(0, 2, 0, 11.0), (1, 2, 1, 11.0)]
