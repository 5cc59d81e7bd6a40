"""Serving loop front end: continuous batching over the C ABI.

`Server` starts the library's worker (sp_serve_start) on a SpiralGPU
context.  `submit` returns a Ticket at once; the worker coalesces queued
requests into batches and overlaps batches on separate lanes (streams).
`Ticket.result()` blocks in the library (GIL released) until the response
bytes are written.

`poisson_load` drives a Server with seeded Poisson arrivals and reports
throughput and server-side latency percentiles (arrival -> response ready,
timed by the library: sp_wait_timed).  `single_query_loop` serves the same
arrivals with the plain single-query path (one sp_answer at a time, first
come first served), the baseline the batching server is compared with.
"""
from __future__ import annotations

import ctypes
import threading
import time

import numpy as np

from .lib import SpiralError, SpiralGPU, SpRequest, _check, _P, _U64, _I


class Ticket:
    def __init__(self, server: "Server", tid: int, response: np.ndarray, query: np.ndarray, t_submit: float):
        self.server = server
        self.id = tid
        self.response = response
        self._query = query          # kept alive until submission copied it
        self.t_submit = t_submit
        self.t_done = None
        self.server_ms = None        # submit -> response written, measured by the library
        self.status = None

    def done(self) -> bool:
        if self.status is not None:
            return True
        d, st = _I(), _I()
        _check(self.server.gpu.lib.sp_poll(self.server.gpu.h, self.id, ctypes.byref(d), ctypes.byref(st)))
        if d.value:
            self.status = st.value
            self.t_done = time.perf_counter()
        return bool(d.value)

    def result(self) -> np.ndarray:
        if self.status is None:
            st, ms = _I(), ctypes.c_double()
            _check(self.server.gpu.lib.sp_wait_timed(self.server.gpu.h, self.id, ctypes.byref(st), ctypes.byref(ms)))
            self.status = st.value
            self.server_ms = ms.value
            self.t_done = time.perf_counter()
        if self.status != 0:
            raise SpiralError(self.status, f"request {self.id} failed")
        return self.response


class Server:
    """Continuous-batching server over a SpiralGPU context."""

    def __init__(self, gpu: SpiralGPU, lanes: int = 2):
        self.gpu = gpu
        _check(gpu.lib.sp_serve_start(gpu.h, lanes))
        self.lanes = lanes

    def submit(self, client_id: int, db_id: int, query: np.ndarray) -> Ticket:
        q = np.ascontiguousarray(query, dtype=np.uint64)
        resp = np.empty(self.gpu.response_bytes, dtype=np.uint8)
        req = SpRequest(client_id, db_id, q.ctypes.data, resp.ctypes.data, resp.nbytes, 0)
        t = _U64()
        now = time.perf_counter()
        _check(self.gpu.lib.sp_submit(self.gpu.h, ctypes.byref(req), ctypes.byref(t)))
        return Ticket(self, t.value, resp, q, now)

    def stats(self) -> dict:
        a, b, c = _U64(), _U64(), _U64()
        _check(self.gpu.lib.sp_serve_stats(self.gpu.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return {"served": a.value, "batches": b.value, "queued": c.value}

    def stop(self) -> None:
        if self.gpu.h:
            _check(self.gpu.lib.sp_serve_stop(self.gpu.h))

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.stop()


def poisson_load(server: Server, requests: list, rate_qps: float, seed: int = 0) -> dict:
    """Submit `requests` [(client, db, query), ...] with exponential
    inter-arrival times at `rate_qps`; wait for all; returns qps and
    latency percentiles (ms) and the responses in request order."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate_qps, size=len(requests))
    tickets = []
    t0 = time.perf_counter()
    next_t = t0
    for (cid, did, q), g in zip(requests, gaps):
        next_t += g
        while True:
            now = time.perf_counter()
            if now >= next_t:
                break
            time.sleep(min(next_t - now, 0.0005))
        tickets.append(server.submit(cid, did, q))
    outs = [t.result() for t in tickets]
    # completion instants from the library's own clock (the Python side only
    # collects the tickets after the last submission)
    t_end = max(t.t_submit + t.server_ms / 1e3 for t in tickets)
    lat = np.array([t.server_ms for t in tickets])
    return {"offered_qps": rate_qps, "achieved_qps": len(requests) / (t_end - t0),
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_ms": float(lat.mean()), "n": len(requests), "responses": outs}


def single_query_loop(gpu: SpiralGPU, requests: list, rate_qps: float, seed: int = 0) -> dict:
    """The plain single-query server under the arrivals of poisson_load with
    the same seed: requests are answered one at a time in arrival order
    through sp_answer; latency is arrival -> response returned (host clock)."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate_qps, size=len(requests))
    arrivals = np.cumsum(gaps)
    out = np.empty(gpu.response_bytes, dtype=np.uint8)
    outs, lat = [], []
    t0 = time.perf_counter()
    for (cid, did, q), a in zip(requests, arrivals):
        while True:
            now = time.perf_counter() - t0
            if now >= a:
                break
            time.sleep(min(a - now, 0.0005))
        gpu.answer(cid, did, q, out=out)
        lat.append((time.perf_counter() - t0 - a) * 1e3)
        outs.append(out.copy())
    t_end = time.perf_counter() - t0
    lat = np.array(lat)
    return {"offered_qps": rate_qps, "achieved_qps": len(requests) / t_end,
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_ms": float(lat.mean()), "n": len(requests), "responses": outs}


__all__ = ["Server", "Ticket", "poisson_load", "single_query_loop", "threading"]
