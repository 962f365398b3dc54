"""Serving engine: job results against the FP64 oracle (spectra put by the
caller), and the same job alone and inside a concurrent mix (other sizes,
deltas, methods and a PWS job) giving identical NCFs.

Tolerance: NCF rows relative L2 1e-5 (plain and tensor), PWS rows 1e-5;
alone vs mix: bit-identical (every kernel is deterministic and a job's
result depends only on its spectra)."""

import numpy as np
import pytest

from oracle import stack_oracle as sto
from oracle import xc_oracle as xo

pytestmark = pytest.mark.gpu


def rel_rows(a, b):
    return np.linalg.norm(a - b, axis=-1) / np.maximum(np.linalg.norm(b, axis=-1), 1e-30)


def job_pairs(nsta):
    src, rec = [], []
    for a in range(nsta):
        for b in range(a + 1, nsta):
            for i in range(3):
                for j in range(3):
                    src.append(3 * a + i)
                    rec.append(3 * b + j)
    return np.array(src), np.array(rec)


@pytest.fixture(scope="module")
def server(built_lib, torch_cuda):
    from fastxc_gb300.serve import Server

    s = Server(slots=3, cache_gib=2.0, work_gib=6.0, chunk_gib=0.25, synthetic=False, keep_results=True)
    yield s
    s.close()


def put_days(server, rng, stations, days, delta):
    nspec, nstep = server.geometry(delta)
    spec = {}
    for st in stations:
        for d in days:
            x = (rng.standard_normal((nstep, 3, nspec)) + 1j * rng.standard_normal((nstep, 3, nspec))).astype(np.complex64)
            server.put_spectra(st, d, delta, x)
            spec[(st, d)] = x
    return spec, nspec, nstep


@pytest.mark.parametrize("method", [0, 1], ids=["plain", "tensor"])
def test_job_matches_oracle(server, method):
    rng = np.random.default_rng(5 + method)
    delta, lag = 0.2, 100.0
    stations, days = [40 + method, 7, 19], [3, 4]
    spec, nspec, nstep = put_days(server, rng, stations, days, delta)
    jid = server.submit(stations, 3, 2, delta, lag, method=method)
    info = server.wait(jid, timeout_s=300.0)
    got = server.fetch(jid, info)
    server.release(jid)
    # oracle over the job's channels: station order of the job, both days' windows
    y = np.concatenate([np.concatenate([spec[(st, d)] for st in stations], axis=1) for d in days], axis=0)
    src, rec = job_pairs(len(stations))
    ref = xo.xc_run(y, src, rec, 1.0 / (2 * nstep), xo.finalize_shape(nspec, nstep, delta, lag))
    assert got.shape == ref.shape == (27, info.cc_size)
    assert rel_rows(got, ref).max() < 1e-5


def test_pws_job_matches_oracle(server):
    rng = np.random.default_rng(9)
    delta, lag, power = 0.2, 60.0, 2.0
    stations, days = [101, 102], [0, 1, 2]
    spec, nspec, nstep = put_days(server, rng, stations, days, delta)
    jid = server.submit(stations, 0, 3, delta, lag, method=0, pws=True, pws_power=power)
    info = server.wait(jid, timeout_s=300.0)
    lin, pws = server.fetch(jid, info, pws=True)
    server.release(jid)
    src, rec = job_pairs(2)
    shape = xo.finalize_shape(nspec, nstep, delta, lag)
    per_day = np.stack([xo.xc_run(np.concatenate([spec[(st, d)] for st in stations], axis=1), src, rec,
                                  1.0 / nstep, shape) for d in days], axis=1)  # [pair][day][cc]
    assert rel_rows(lin, per_day.mean(axis=1)).max() < 1e-5
    ref = np.stack([sto.pws(per_day[p], 1, power) for p in range(per_day.shape[0])])
    assert rel_rows(pws, ref).max() < 1e-5


def test_same_result_alone_and_in_mix(built_lib, torch_cuda):
    from fastxc_gb300.serve import Server

    s = Server(slots=3, cache_gib=4.0, work_gib=12.0, chunk_gib=0.5, synthetic=True, seed=3, keep_results=True)
    try:
        a = dict(stations=[11, 3, 250, 77], day0=2, ndays=3, delta=0.1, lag=120.0, method=1)
        jid = s.submit(**a)
        alone = s.fetch(jid, s.wait(jid, timeout_s=300.0))
        s.release(jid)
        mix = [
            dict(stations=list(range(300, 330)), day0=0, ndays=2, delta=0.1, lag=200.0, method=1),
            a,
            dict(stations=[5, 6, 7], day0=1, ndays=4, delta=0.2, lag=50.0, method=0, pws=True),
            dict(stations=[11, 3], day0=2, ndays=1, delta=0.05, lag=200.0, method=0),
            dict(stations=list(range(20, 60)), day0=3, ndays=1, delta=0.2, lag=100.0, method=-1),
            a,
        ]
        ids = [s.submit(**m) for m in mix]
        infos = [s.wait(i, timeout_s=300.0) for i in ids]
        for i in (1, 5):
            again = s.fetch(ids[i], infos[i])
            assert np.array_equal(again, alone)
        # the 20 Hz job (nfft above the one-CTA transform) completes with finite NCFs
        d = s.fetch(ids[3], infos[3])
        assert infos[3].cc_size == 8001 and np.isfinite(d).all() and np.abs(d).max() > 0
        st = s.stats()
        assert st.jobs_done == 7 and st.queued == 0 and st.work_used_bytes == 0
        for i in ids:
            s.release(i)
    finally:
        s.close()
