"""Multi-rank sharding logic on CPU ranks (gloo, world size 2).

Each rank computes its shard with the FP64 oracle standing in for the GPU
engine (same infer() shape), then the ranks gather the global category set,
which must equal the single-process result.  A rank that fails before the
gather makes the others raise instead of hanging.
"""
import os
import socket

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


class OracleEngine:
    def __init__(self, layers, N, bias):
        self.layers, self.N, self.bias = layers, N, bias

    def infer(self, Y0):
        from oracle import oracle as orc
        _, alive, _ = orc.infer(self.layers, self.N, self.bias, Y0, precision=64, want_y=False)
        return alive, np.flatnonzero(alive).astype(np.int32)


def _worker(rank, world, port, total, fail_rank, q):
    import sys
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import snicit_gb300 as sg
    from snicit_gb300 import shard
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import datetime
    dist.init_process_group("gloo", rank=rank, world_size=world,
                            timeout=datetime.timedelta(seconds=20))
    try:
        N, L = 128, 6
        layers = [sg.generate_layer_csr(N, 3, l) for l in range(L)]
        eng = OracleEngine(layers, N, -0.3)
        if rank == fail_rank:
            raise RuntimeError("injected failure before the gather")
        ids = shard.run_shard(eng, lambda o, c: sg.generate_inputs(N, 3, o, c), total, rank, world)
        q.put((rank, "ok", ids.tolist()))
    except Exception as ex:  # reported to the parent
        q.put((rank, "error", repr(ex)))
    finally:
        try:
            dist.destroy_process_group()
        except Exception:
            pass


def _spawn(world, total, fail_rank=-1):
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, world, port, total, fail_rank, q)) for r in range(world)]
    for p in ps:
        p.start()
    out = [q.get(timeout=120) for _ in ps]
    for p in ps:
        p.join(timeout=60)
        if p.is_alive():
            p.kill()
    return sorted(out)


def test_shard_ranges_cover_rows():
    from snicit_gb300.shard import shard_range
    for total in (0, 1, 7, 60000):
        for world in (1, 2, 3, 8):
            spans = [shard_range(total, world, r) for r in range(world)]
            assert spans[0][0] == 0
            for (o1, c1), (o2, _) in zip(spans, spans[1:]):
                assert o1 + c1 == o2
            assert sum(c for _, c in spans) == total
            assert max(c for _, c in spans) - min(c for _, c in spans) <= 1
    with pytest.raises(ValueError):
        shard_range(5, 2, 2)


def test_two_ranks_gather_equals_single_process():
    import snicit_gb300 as sg
    from oracle import oracle as orc
    total = 301
    out = _spawn(2, total)
    assert [o[1] for o in out] == ["ok", "ok"], out
    N, L = 128, 6
    layers = [sg.generate_layer_csr(N, 3, l) for l in range(L)]
    _, alive, _ = orc.infer(layers, N, -0.3, sg.generate_inputs(N, 3, 0, total), precision=64,
                            want_y=False)
    want = np.flatnonzero(alive).tolist()
    assert out[0][2] == want and out[1][2] == want


def test_failed_rank_is_reported_not_hung():
    out = _spawn(2, 50, fail_rank=1)
    status = {r: s for r, s, _ in out}
    assert status[1] == "error"
    assert status[0] == "error"  # the gather sees the dead peer and raises
