"""ctypes mirror of the serving engine (fxc_server_* in include/fastxc_gb300.h)
and the Poisson job-stream driver used by the serving benchmark."""

from __future__ import annotations

import ctypes as C
import threading
import time

import numpy as np

from . import _lib


from ._lib import Job, JobInfo, ServerConfig, ServerStats  # noqa: E402


class Server:
    def __init__(self, device=0, slots=4, cache_gib=32.0, work_gib=64.0, chunk_gib=4.0, synthetic=True, seed=0,
                 win_len=3600.0, lag_max=200.0, max_wait_s=5.0, keep_results=True):
        self.L = _lib.lib()
        cfg = ServerConfig(device, slots, cache_gib, work_gib, chunk_gib, int(synthetic), seed, win_len, lag_max,
                           max_wait_s, int(keep_results))
        self.h = C.c_void_p()
        self.L.fxc_server_create(C.byref(cfg), C.byref(self.h))

    def close(self):
        if self.h:
            self.L.fxc_server_destroy(self.h)
            self.h = C.c_void_p()

    def geometry(self, delta: float):
        nspec, nstep = C.c_int32(), C.c_int32()
        self.L.fxc_server_geometry(self.h, delta, C.byref(nspec), C.byref(nstep))
        return nspec.value, nstep.value

    def put_spectra(self, station: int, day: int, delta: float, spec: np.ndarray):
        spec = np.ascontiguousarray(spec, np.complex64)
        self.L.fxc_server_put_spectra(self.h, station, day, delta, spec.ctypes.data_as(C.c_void_p))

    def submit(self, stations, day0, ndays, delta, lag, method=1, pws=False, pws_power=1.0) -> int:
        st = np.ascontiguousarray(stations, np.int32)
        job = Job(st.ctypes.data_as(C.POINTER(C.c_int32)), st.size, day0, ndays, delta, lag, method, int(pws),
                  pws_power)
        jid = C.c_int64()
        self.L.fxc_server_submit(self.h, C.byref(job), C.byref(jid))
        return jid.value

    def wait(self, jid: int, timeout_s: float = 0.0) -> JobInfo:
        info = JobInfo()
        self.L.fxc_server_wait(self.h, jid, timeout_s, C.byref(info))
        return info

    def fetch(self, jid: int, info: JobInfo, pws=False):
        ncf = np.empty((info.npairs, info.cc_size), np.float32)
        out = np.empty_like(ncf) if pws else None
        self.L.fxc_server_fetch(self.h, jid, ncf.ctypes.data_as(C.c_void_p),
                                out.ctypes.data_as(C.c_void_p) if pws else None)
        return (ncf, out) if pws else ncf

    def release(self, jid: int):
        self.L.fxc_server_release(self.h, jid)

    def stats(self) -> ServerStats:
        s = ServerStats()
        self.L.fxc_server_stats(self.h, C.byref(s))
        return s


def poisson_stream(server: Server, seconds: float, rate: float, seed: int = 0, pool: int = 1000,
                   sta_range=(2, 200), day_range=(1, 30), deltas=(0.05, 0.1, 0.2), lag_range=(50.0, 200.0),
                   pws_frac=0.1, days_total=60, method=-1, wait_limit_s=600.0):
    """Submits a Poisson stream of jobs for `seconds` (mean `rate` per s) and
    waits for all of them (each at most wait_limit_s). Returns (per-job
    records, wall seconds from the first submission to the last result,
    failure messages)."""
    rng = np.random.default_rng(seed)
    t = 0.0
    plan = []
    while True:
        t += rng.exponential(1.0 / rate)
        if t > seconds:
            break
        nsta = int(rng.integers(sta_range[0], sta_range[1] + 1))
        ndays = int(rng.integers(day_range[0], day_range[1] + 1))
        plan.append(dict(at=t, stations=rng.choice(pool, nsta, replace=False).astype(np.int32),
                         day0=int(rng.integers(0, days_total - ndays + 1)), ndays=ndays,
                         delta=float(rng.choice(deltas)), lag=float(rng.uniform(*lag_range)),
                         pws=bool(rng.random() < pws_frac)))
    records = []
    failures = []
    lock = threading.Lock()

    def waiter(jid, job):
        try:
            info = server.wait(jid, timeout_s=wait_limit_s)
            server.release(jid)
        except Exception as e:  # timed out or failed: reported, not raised
            with lock:
                failures.append(str(e))
            return
        with lock:
            records.append(dict(latency=info.end_s - info.submit_s, queue=info.start_s - info.submit_s,
                                pair_windows=info.pair_windows, npairs=info.npairs, delta=job["delta"],
                                nsta=len(job["stations"]), ndays=job["ndays"], pws=job["pws"], end=info.end_s,
                                submit=info.submit_s))

    threads = []
    t0 = time.perf_counter()
    for job in plan:
        dt = job["at"] - (time.perf_counter() - t0)
        if dt > 0:
            time.sleep(dt)
        try:
            jid = server.submit(job["stations"], job["day0"], job["ndays"], job["delta"], job["lag"], method=method,
                                pws=job["pws"])
        except Exception as e:
            failures.append(f"submit: {e}")
            continue
        th = threading.Thread(target=waiter, args=(jid, job), daemon=True)
        th.start()
        threads.append(th)
    for th in threads:
        th.join()
    wall = max(r["end"] for r in records) - min(r["submit"] for r in records) if records else 0.0
    return records, wall, failures
