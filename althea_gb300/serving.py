"""Probe re-bake serving over the native server (althea_ibl_server_*).

``ProbeServer`` owns one server: requests carry host (pinned) env maps, or
name a map registered with the server (resident on the device) plus the sun
lobes to add to it, and host output buffers; the server admits them by slot
and HBM budget, overlaps their work on the device and reports completion
times on its steady clock.  ``run_poisson`` replays a Poisson arrival stream
against a server and returns latency percentiles and throughput.
"""
from __future__ import annotations

import ctypes
import time
from dataclasses import dataclass
from typing import Dict, List

import numpy as np

from . import ibl


@dataclass
class RequestBuffers:
    env: object            # pinned (H, W, 4) float32 host tensor, or None (resident map)
    mips: object           # pinned flat float32 host tensor (all mips back to back)
    irradiance: object     # pinned (ih, iw, 4) float32 host tensor
    mip_sizes: List[tuple]
    env_id: int = 0        # a map registered with the server, or 0
    env_size: tuple = (0, 0)   # (W, H) of the env map


def mip_sizes_for(w: int, h: int, mip_count: int) -> List[tuple]:
    fw, fh = max(w >> 1, 1), max(h >> 1, 1)
    return [(max(fw >> m, 1), max(fh >> m, 1)) for m in range(mip_count)]


class ProbeServer:
    def __init__(self, budget_bytes: int, max_inflight: int = 8, samples: int = 1024,
                 generator: int = ibl.GEN_HAMMERSLEY, irradiance_size=(32, 16),
                 path: int = ibl.PATH_PLAIN):
        self.cfg = ibl.ServerConfig(budget_bytes, max_inflight, samples, generator,
                                    irradiance_size[0], irradiance_size[1], path)
        self.irradiance_size = irradiance_size
        self._s = ctypes.c_void_p()
        ibl._check(ibl.load().althea_ibl_server_create(ctypes.byref(self.cfg),
                                                       ctypes.byref(self._s)))
        # Each submission gets its own tag inside the native server, mapped back
        # to the caller's tag on completion; its buffers are referenced here
        # until then, so they stay alive while the device reads and writes them.
        self._inflight: Dict[int, tuple] = {}
        self._resident: Dict[int, tuple] = {}
        self._next = 0
        self._done = (ibl.Completion * 256)()

    def buffers(self, env_np: np.ndarray, mip_count: int) -> RequestBuffers:
        """Pinned host buffers for one request (env copied in)."""
        import torch
        h, w = env_np.shape[:2]
        env = torch.from_numpy(np.ascontiguousarray(env_np)).pin_memory()
        sizes = mip_sizes_for(w, h, mip_count)
        mips = torch.empty(sum(a * b * 4 for a, b in sizes), dtype=torch.float32).pin_memory()
        iw, ih = self.irradiance_size
        irr = torch.empty((ih, iw, 4), dtype=torch.float32).pin_memory()
        return RequestBuffers(env, mips, irr, sizes, 0, (w, h))

    def register_env(self, env) -> int:
        """Uploads an (H, W, 4) float32 map (numpy, host or CUDA tensor) once;
        it stays on the device, counted against the budget.  Returns its id."""
        import torch
        t = env if isinstance(env, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(env))
        t = t.contiguous()
        if t.dtype != torch.float32 or t.dim() != 3 or t.shape[2] != 4:
            raise ibl.IBLError(ibl.ERR_INVALID_ARGUMENT, "env must be (H, W, 4) float32")
        h, w = t.shape[:2]
        out = ctypes.c_int()
        ibl._check(ibl.load().althea_ibl_server_register_env(
            self._s, t.data_ptr(), w, h, 1 if t.is_cuda else 0, ctypes.byref(out)))
        self._resident[out.value] = (w, h)
        return out.value

    def unregister_env(self, env_id: int) -> None:
        ibl._check(ibl.load().althea_ibl_server_unregister_env(self._s, env_id))
        self._resident.pop(env_id, None)

    def output_buffers(self, env_id: int, mip_count: int) -> RequestBuffers:
        """Pinned host outputs for requests on a resident map (no env buffer)."""
        import torch
        w, h = self._resident[env_id]
        sizes = mip_sizes_for(w, h, mip_count)
        mips = torch.empty(sum(a * b * 4 for a, b in sizes), dtype=torch.float32).pin_memory()
        iw, ih = self.irradiance_size
        irr = torch.empty((ih, iw, 4), dtype=torch.float32).pin_memory()
        return RequestBuffers(None, mips, irr, sizes, env_id, (w, h))

    def submit(self, tag: int, buf: RequestBuffers, suns=()) -> None:
        """Queues a re-bake into buf's outputs -- of buf.env, or of the resident
        map buf.env_id -- with the given sun lobes [(direction, sigma rad,
        radiance), ...] added on the device first.  Its completion is reported
        by poll() under `tag` (tags may repeat)."""
        if buf.env is not None:
            h, w = buf.env.shape[:2]
        else:
            w, h = buf.env_size
        key = self._next
        req = ibl.Request()
        req.env_host = buf.env.data_ptr() if buf.env is not None else None
        req.env_width, req.env_height = w, h
        req.mip_count = len(buf.mip_sizes)
        req.irradiance_host = buf.irradiance.data_ptr()
        req.mips_host = buf.mips.data_ptr()
        req.tag = key
        req.env_id = buf.env_id
        arr, n = ibl.make_suns(suns)
        req.sun_count = n
        req.suns = arr
        ibl._check(ibl.load().althea_ibl_server_submit(self._s, ctypes.byref(req)))
        self._next += 1
        self._inflight[key] = (tag, buf)

    def poll(self) -> List[ibl.Completion]:
        n = ctypes.c_int()
        out = []
        while True:
            ibl._check(ibl.load().althea_ibl_server_poll(self._s, self._done, len(self._done),
                                                         ctypes.byref(n)))
            for k in range(n.value):
                c = self._done[k]
                tag, _ = self._inflight.pop(c.tag, (c.tag, None))  # buffers free again
                out.append(ibl.Completion(tag, c.status, c.submit_s, c.start_s, c.done_s))
            if n.value < len(self._done):
                return out

    def stats(self) -> ibl.ServerStats:
        st = ibl.ServerStats()
        ibl._check(ibl.load().althea_ibl_server_get_stats(self._s, ctypes.byref(st)))
        return st

    def request_bytes(self, w: int, h: int, mip_count: int) -> int:
        return ibl.load().althea_ibl_server_request_bytes(self._s, w, h, mip_count)

    def drain(self, timeout_s: float = 120.0) -> List[ibl.Completion]:
        out = []
        t0 = time.monotonic()
        while True:
            out += self.poll()
            st = self.stats()
            if st.inflight == 0 and st.queued == 0:
                return out + self.poll()
            if time.monotonic() - t0 > timeout_s:
                raise TimeoutError("server did not drain")
            time.sleep(0.0002)

    def close(self) -> None:
        if self._s:
            ibl.load().althea_ibl_server_destroy(self._s)
            self._s = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def now() -> float:
    return ibl.load().althea_ibl_server_now()


def run_poisson(server: ProbeServer, pool: List[RequestBuffers], rate: float, n_requests: int,
                seed: int = 0, suns_for=None) -> dict:
    """Submits n_requests at Poisson arrival times (rate per second), cycling
    through the prepared request buffers, and returns latency statistics.
    suns_for(i): the sun lobes of request i (added on the device), or None.
    Latency = completion (host callback on the request's stream) - arrival."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, size=n_requests)
    arrivals = np.cumsum(gaps)
    t0 = now()
    done: Dict[int, ibl.Completion] = {}
    arrival_abs = {}
    in_use = {}  # pool slot -> tag using it (a buffer is reused only after it completes)
    for i in range(n_requests):
        target = t0 + arrivals[i]
        k = i % len(pool)
        while True:
            for c in server.poll():
                done[c.tag] = c
                in_use = {s: t for s, t in in_use.items() if t != c.tag}
            if now() >= target and k not in in_use:
                break
            time.sleep(0.00005)
        arrival_abs[i] = target
        in_use[k] = i
        server.submit(i, pool[k], suns_for(i) if suns_for is not None else ())
    for c in server.drain():
        done[c.tag] = c
    t_end = max(c.done_s for c in done.values())
    lat = np.array([done[i].done_s - arrival_abs[i] for i in range(n_requests)
                    if done[i].status == ibl.OK])
    st = server.stats()
    return {"rate": rate, "requests": n_requests, "ok": int(len(lat)),
            "p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
            "mean_ms": float(lat.mean() * 1e3),
            "throughput": n_requests / (t_end - t0),
            "peak_bytes": int(st.peak_bytes_in_use)}
