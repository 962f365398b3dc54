"""FP64 restatement of the xc_fast stage (correlation, within-window stack,
inverse FFT, lag cut) and of its integer work (jobs, tasks, path table).

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

Pinning: the integer functions (``finalize_shape``, ``build_jobs``,
``build_tasks_for_job``, path-table lookups) follow the reference C/C++ line by
line and are checked bit-exactly against the reference's own scheduler and
path-table code compiled for the CPU (``oracle/build_ref.py``). The
reference ships no golden NCF vectors and its correlation runs only on a GPU
through cuFFT, so the float path (accumulateStepXc2DKernel,
native/xc/kernels/cuda.kernels.cu:16-36, and finalize_xc_batch,
native/xc/worker/executor.cu:6-55) is "parity unpinned" beyond this FP64
restatement.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

# ---------------------------------------------------------------------------
# Shape: native/xc/io/input.cu:1033-1054 (finalize_shape)
# ---------------------------------------------------------------------------


@dataclass(frozen=True)
class XcShape:
    nspec: int
    nstep: int
    nfft: int
    half_cc: int
    cc_size: int
    dt: float


def _llround(x: float) -> int:
    # C llround: half away from zero
    return int(np.sign(x) * np.floor(abs(x) + 0.5))


def finalize_shape(nspec: int, nstep: int, dt: float, cc_length: float) -> XcShape:
    """native/xc/io/input.cu:1033-1054. dt and cc_length are float32 values."""
    dt32 = float(np.float32(dt))
    cc32 = float(np.float32(cc_length))
    if nspec < 2 or nstep <= 0 or dt32 <= 0.0 or cc32 <= 0.0:
        raise ValueError("invalid shape")
    nfft = 2 * (nspec - 1)
    half_cc = _llround(cc32 / dt32)
    if half_cc >= nspec:
        half_cc = nspec - 1
    cc_size = 2 * half_cc + 1
    if cc_size <= 0 or cc_size > nfft:
        raise ValueError("invalid cc_size")
    return XcShape(nspec, nstep, nfft, half_cc, cc_size, dt32)


# ---------------------------------------------------------------------------
# Correlation + stack: native/xc/kernels/cuda.kernels.cu:16-36 and the step
# loop native/xc/worker/async_workers.cu:61-83 (scale = 1/nstep applied to
# every step's product before accumulation).
# ---------------------------------------------------------------------------


def xc_stack(spec: np.ndarray, src: np.ndarray, rec: np.ndarray, scale: float,
             mask: np.ndarray | None = None) -> np.ndarray:
    """spec: [nwin][nchan][nspec] complex; returns [npairs][nspec] complex128.

    stack[p] = sum_w scale * conj(spec[w, src[p]]) * spec[w, rec[p]]
    A window with mask[w, ch] == 0 contributes zero for that channel.
    """
    spec = np.asarray(spec)
    nwin = spec.shape[0]
    src = np.asarray(src, dtype=np.int64)
    rec = np.asarray(rec, dtype=np.int64)
    out = np.zeros((src.size, spec.shape[2]), dtype=np.complex128)
    for w in range(nwin):
        s = spec[w].astype(np.complex128)
        if mask is not None:
            s = s * (np.asarray(mask[w]) != 0)[:, None]
        out += scale * (np.conj(s[src]) * s[rec])
    return out


def xc_finalize(stack: np.ndarray, shape: XcShape) -> np.ndarray:
    """native/xc/worker/executor.cu:6-55.

    (-1)^f phase shift (applyPhaseShiftKernel, cuda.kernels.cu:38-49) ->
    C2R of length nfft (imaginary parts of DC/Nyquist ignored, as C2R does)
    -> x 1/(nfft*dt) (InvNormalize2DKernel, cuda.kernels.cu:51-62) -> keep
    cc_size samples from index nspec-half_cc-1 (= nfft/2 - half_cc).
    """
    stack = np.asarray(stack, dtype=np.complex128)
    f = np.arange(shape.nspec)
    sgn = np.where(f % 2 == 0, 1.0, -1.0)
    x = np.fft.irfft(stack * sgn, n=shape.nfft, axis=-1) * shape.nfft  # unnormalised C2R
    wdt = float(np.float32(np.float32(shape.nfft) * np.float32(shape.dt)))
    x = x * (1.0 / wdt)
    start = shape.nspec - shape.half_cc - 1
    return x[..., start:start + shape.cc_size]


def xc_run(spec, src, rec, scale, shape: XcShape, mask=None) -> np.ndarray:
    return xc_finalize(xc_stack(spec, src, rec, scale, mask), shape)


# ---------------------------------------------------------------------------
# Allowed path table: native/xc/io/path_table.c
# ---------------------------------------------------------------------------


def make_allowed_path_id(src_gnsl: int, rec_gnsl: int) -> int:
    """path_table.c:9-17."""
    if src_gnsl <= 0 or src_gnsl > 9999 or rec_gnsl <= 0 or rec_gnsl > 9999:
        return -1
    return src_gnsl * 10000 + rec_gnsl


def canonical_gnsl_pair(a: int, b: int) -> tuple[int, int]:
    """path_table.c:19-36."""
    return (a, b) if a <= b else (b, a)


def find_allowed_path_canonical(path_ids: set[int] | dict, a: int, b: int):
    """path_table.c:188-202: returns the path id if present, else None."""
    s, r = canonical_gnsl_pair(a, b)
    pid = make_allowed_path_id(s, r)
    if pid <= 0:
        return None
    return pid if pid in path_ids else None


# ---------------------------------------------------------------------------
# Jobs and tasks: native/xc/worker/scheduler.cu:43-167
# ---------------------------------------------------------------------------

ROW_TARGET_BLOCKS = 1  # native/xc/runtime.hpp:26 (kRowTargetBlocks)


@dataclass(frozen=True)
class RowBatchJob:
    anchor_block: int
    target_begin_block: int
    target_end_block: int
    block_size: int
    file_count: int
    anchor_begin: int
    anchor_end: int
    target_begin: int
    target_end: int


def _fill_row_job(file_count, block_size, anchor, tb, te) -> RowBatchJob:
    """scheduler.cu:25-41."""
    ab = anchor * block_size
    return RowBatchJob(anchor, tb, te, block_size, file_count, ab,
                       min(file_count, ab + block_size), tb * block_size,
                       min(file_count, te * block_size))


def build_jobs(file_count: int, block_size: int) -> list[RowBatchJob]:
    """scheduler.cu:43-63."""
    jobs = []
    block_count = (file_count + block_size - 1) // block_size
    for anchor in range(block_count):
        jobs.append(_fill_row_job(file_count, block_size, anchor, anchor, anchor + 1))
        target = anchor + 1
        while target < block_count:
            te = min(block_count, target + ROW_TARGET_BLOCKS)
            jobs.append(_fill_row_job(file_count, block_size, anchor, target, te))
            target += ROW_TARGET_BLOCKS
    return jobs


@dataclass(frozen=True)
class XcTask:
    src_meta_idx: int
    rec_meta_idx: int
    src_local_idx: int
    rec_local_idx: int
    path_id: int
    is_autocorr: bool


def build_tasks_for_job(gnsl_ids: list[int], path_ids, job: RowBatchJob):
    """scheduler.cu:65-148. gnsl_ids[i] is the NSL id of channel i (the
    stable-sorted NSLC order of the timestamp). Returns (tasks, loaded)."""
    loaded = list(range(job.anchor_begin, job.anchor_end))
    if job.target_begin != job.anchor_begin:
        loaded += list(range(job.target_begin, job.target_end))

    def local_idx(m):
        if job.anchor_begin <= m < job.anchor_end:
            return m - job.anchor_begin
        return (job.anchor_end - job.anchor_begin) + (m - job.target_begin)

    tasks: list[XcTask] = []

    def push(s, r, pid, auto):
        tasks.append(XcTask(s, r, local_idx(s), local_idx(r), pid, auto))

    def try_pair(a, b, same_block):
        ga, gb = gnsl_ids[a], gnsl_ids[b]
        auto = ga == gb
        if same_block and not auto and b <= a:
            return
        pid = find_allowed_path_canonical(path_ids, ga, gb)
        if pid is None:
            return
        if auto:
            push(a, b, pid, True)
            if not same_block:
                push(b, a, pid, True)
            return
        if ga < gb:
            push(a, b, pid, False)
        else:
            push(b, a, pid, False)

    for tb in range(job.target_begin_block, job.target_end_block):
        begin = tb * job.block_size
        end = min(job.file_count, begin + job.block_size)
        same = tb == job.anchor_block
        if same:
            begin, end = job.anchor_begin, job.anchor_end
        for a in range(job.anchor_begin, job.anchor_end):
            for b in range(begin, end):
                try_pair(a, b, same)
    return tasks, loaded
