"""Request server (continuous batching) over the C ABI, and the sparse-MLP
serving workload.

Server binds sdnn_server_* (include/snicit_gb300.h): requests of any size up
to the slot capacity are submitted at any time, admitted into free slots in
arrival order, and their results (category flags, dense-head logits and
argmax, latency) collected by id.

sparse_mlp() builds the serving network: 1024 inputs uniform in [0, 1],
hidden layers of width 1024 with Bernoulli(3%) weights drawn N(0, 0.3^2),
bias -0.05, clamp 32, then a dense 1024 x 10 head -- the shape of the
reference's beyond nets (src/beyond/general.hpp:36-102) at the serving sizes.
"""
import ctypes
from dataclasses import dataclass

import numpy as np

from ._lib import ServerConfig, ServerStats, SdnnError, check, load
from .engine import coo_to_csr


@dataclass
class Result:
    flags: np.ndarray
    logits: np.ndarray
    argmax: np.ndarray
    latency_s: float


class Server:
    def __init__(self, engine, head_w=None, head_b=None, slots=2, max_rows=16384,
                 memory_fraction=0.25, max_pending=1 << 16, max_delay_us=0,
                 max_requests_per_pass=0):
        lib = load()
        cfg = ServerConfig()
        check(lib.sdnn_server_config_default(ctypes.byref(cfg)))
        cfg.slots = slots
        cfg.max_rows = max_rows
        cfg.memory_fraction = memory_fraction
        cfg.max_pending = max_pending
        cfg.max_delay_us = max_delay_us
        cfg.max_requests_per_pass = max_requests_per_pass
        self.N = engine.N
        self.H = 0 if head_w is None else int(np.shape(head_w)[1])
        cfg.head_outputs = self.H
        hw = hb = None
        if self.H:
            hw = np.ascontiguousarray(head_w, dtype=np.float32)
            hb = np.ascontiguousarray(head_b, dtype=np.float32)
            assert hw.shape == (self.N, self.H) and hb.shape == (self.H,)
        self._h = ctypes.c_void_p()
        self._engine = engine  # the slots read its device weights: keep it alive
        engine._ck(lib.sdnn_server_create(engine._h, ctypes.byref(cfg),
                                          hw.ctypes.data if hw is not None else None,
                                          hb.ctypes.data if hb is not None else None,
                                          ctypes.byref(self._h)))
        self._rows = {}

    @property
    def capacity(self):
        return int(load().sdnn_server_capacity(self._h))

    def submit(self, rows):
        x = np.ascontiguousarray(rows, dtype=np.float32)
        assert x.ndim == 2 and x.shape[1] == self.N
        rid = ctypes.c_uint64(0)
        check(load().sdnn_submit(self._h, x.ctypes.data, x.shape[0], ctypes.byref(rid)))
        self._rows[rid.value] = x.shape[0]
        return rid.value

    def _outputs(self, rid):
        n = self._rows[rid]
        return (np.zeros(n, np.int32), np.zeros((n, self.H), np.float32),
                np.zeros(n, np.int32), ctypes.c_double(0.0))

    def poll(self, rid):
        """Result when finished, else None."""
        f, lg, am, lat = self._outputs(rid)
        done = ctypes.c_int32(0)
        check(load().sdnn_poll(self._h, rid, ctypes.byref(done), f.ctypes.data,
                               lg.ctypes.data if self.H else None,
                               am.ctypes.data if self.H else None, ctypes.byref(lat)))
        if not done.value:
            return None
        del self._rows[rid]
        return Result(f, lg, am, lat.value)

    def wait(self, rid):
        f, lg, am, lat = self._outputs(rid)
        check(load().sdnn_wait(self._h, rid, f.ctypes.data, lg.ctypes.data if self.H else None,
                               am.ctypes.data if self.H else None, ctypes.byref(lat)))
        del self._rows[rid]
        return Result(f, lg, am, lat.value)

    def stats(self):
        s = ServerStats()
        check(load().sdnn_server_get_stats(self._h, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in ServerStats._fields_ if k != "reserved"}

    def close(self):
        if self._h:
            load().sdnn_server_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def sparse_mlp(seed, N=1024, L=120, density=0.03, std=0.3, H=10):
    """Seeded serving network: L CSR layers (N x N, Bernoulli(density) mask,
    N(0, std^2) values) and a dense N x H head (N(0, 1/N) weights, zero bias)."""
    layers = []
    for l in range(L):
        rng = np.random.default_rng([seed, 1, l])
        mask = rng.random((N, N)) < density
        r, c = np.nonzero(mask)
        v = (rng.standard_normal(len(r)) * std).astype(np.float32)
        layers.append(coo_to_csr(N, r, c, v))
    rng = np.random.default_rng([seed, 2])
    head_w = (rng.standard_normal((N, H)) / np.sqrt(N)).astype(np.float32)
    head_b = np.zeros(H, np.float32)
    return layers, head_w, head_b


def mlp_inputs(seed, index, rows, N=1024):
    """Request `index` of the stream: rows x N uniform [0, 1) FP32."""
    return np.random.default_rng([seed, 3, index]).random((rows, N), dtype=np.float32)


def request_stream(seed, count, rate=2000.0, lo=1, hi=4096):
    """Seeded Poisson arrivals (seconds from start) and log-uniform sizes in [lo, hi]."""
    rng = np.random.default_rng([seed, 4])
    arrivals = np.cumsum(rng.exponential(1.0 / rate, count))
    sizes = np.floor(np.exp(rng.uniform(np.log(lo), np.log(hi + 1), count))).astype(np.int64)
    return arrivals, np.clip(sizes, lo, hi)


__all__ = ["Server", "Result", "SdnnError", "sparse_mlp", "mlp_inputs", "request_stream"]
