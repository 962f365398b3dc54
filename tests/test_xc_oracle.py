"""CPU checks of the xc oracle's integer work and shape rules."""

import numpy as np

from oracle import xc_oracle as xo


def test_finalize_shape_config_geometry():
    s = xo.finalize_shape(18523, 24, 0.1, 100.0)
    assert (s.nfft, s.half_cc, s.cc_size) == (37044, 1000, 2001)
    s = xo.finalize_shape(9262, 24, 0.2, 100.0)  # delta 0.2
    assert (s.nfft, s.half_cc, s.cc_size) == (18522, 500, 1001)
    # the cap at nspec-1 gives cc_size = nfft+1, which the reference rejects
    import pytest

    with pytest.raises(ValueError):
        xo.finalize_shape(11, 1, 0.1, 100.0)
    s = xo.finalize_shape(11, 1, 0.1, 0.9)
    assert s.half_cc == 9 and s.cc_size == 19


def test_path_ids():
    assert xo.make_allowed_path_id(12, 345) == 120345
    assert xo.make_allowed_path_id(0, 3) == -1
    assert xo.make_allowed_path_id(10000, 3) == -1
    assert xo.canonical_gnsl_pair(7, 3) == (3, 7)


def test_build_jobs_blocks():
    jobs = xo.build_jobs(10, 4)
    # 3 blocks: (0,0) (0,1) (0,2) (1,1) (1,2) (2,2)
    assert [(j.anchor_block, j.target_begin_block) for j in jobs] == [(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]
    assert jobs[-1].anchor_end == 10 and jobs[2].target_end == 10


def test_tasks_cross_and_auto():
    # 2 stations x 3 components, gnsl 1 and 2; all paths allowed incl. autocorr
    g = [1, 1, 1, 2, 2, 2]
    paths = {10001, 10002, 20002}
    job = xo.build_jobs(6, 6)[0]
    tasks, loaded = xo.build_tasks_for_job(g, paths, job)
    assert loaded == list(range(6))
    pairs = [(t.src_meta_idx, t.rec_meta_idx) for t in tasks]
    # station-1 autocorrelation: all 9 component pairs in row-major order first
    assert pairs[:3] == [(0, 0), (0, 1), (0, 2)]
    assert sum(t.is_autocorr for t in tasks) == 18
    assert sum(not t.is_autocorr for t in tasks) == 9
    # cross pairs have src = lower NSL id
    for t in tasks:
        if not t.is_autocorr:
            assert g[t.src_meta_idx] < g[t.rec_meta_idx]


def test_tasks_cross_block_autocorr_both_orders():
    g = [1, 1, 2, 2]
    paths = {10001}
    jobs = xo.build_jobs(4, 1)
    got = []
    for j in jobs:
        tasks, _ = xo.build_tasks_for_job(g, paths, j)
        got += [(t.src_meta_idx, t.rec_meta_idx) for t in tasks]
    assert got == [(0, 0), (0, 1), (1, 0), (1, 1)]


def test_oracle_stack_is_linear_in_windows():
    rng = np.random.default_rng(0)
    spec = (rng.standard_normal((4, 3, 9)) + 1j * rng.standard_normal((4, 3, 9)))
    src, rec = np.array([0, 1]), np.array([1, 2])
    a = xo.xc_stack(spec[:2], src, rec, 1.0)
    b = xo.xc_stack(spec[2:], src, rec, 1.0)
    c = xo.xc_stack(spec, src, rec, 1.0)
    assert np.allclose(a + b, c)
