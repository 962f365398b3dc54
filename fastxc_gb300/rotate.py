"""ENZ -> RTZ rotation of stacked nine-component NCFs, on the GPU.

Drop-in for fastxc/operators/rotation/python_rotate.py: build_rotate_matrix
(:33-95), rotate_enz_to_rtz (:98-105), rotate_sac_files (:136-182),
rotate_from_lists (:185-199), discover_rotate_list_pairs (:202-211),
rotate_many_from_lists (:219-260), rotate_sourcepack_stack (:263-385) and
rotate_linearstack_sourcepack (:388-393).

The rotation matrices are built exactly as the reference builds them (numpy
float32 scalars), so they are bit-identical; the per-sample 9 x 9 products
run batched over all pairs in fxc_rotate_enz_rtz (FMA in source-component
order), which differs from numpy's matmul only in the float32 summation
order. Geometry comes from the SAC header: Rudoe's geodesic from the event
and station coordinates when all four are set, else the header's own
gcarc/az/baz/dist.
"""

from __future__ import annotations

import concurrent.futures
import csv
import math
import shutil
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from . import sacbin
from .sourcepack import SOURCEPACK_INDEX_HEADER

ENZ_ORDER = ("E-E", "E-N", "E-Z", "N-E", "N-N", "N-Z", "Z-E", "Z-N", "Z-Z")
RTZ_ORDER = ("R-R", "R-T", "R-Z", "T-R", "T-T", "T-Z", "Z-R", "Z-T", "Z-Z")
SAC_COMPONENT_NAMES = ("RR", "RT", "RZ", "TR", "TT", "TZ", "ZR", "ZT", "ZZ")
_FLT_MAX = 3.4028234663852886e38


@dataclass(frozen=True)
class RotateResult:
    input_list: Path
    output_list: Path
    output_paths: tuple
    sample_count: int


def build_rotate_matrix(azimuth_deg: float, back_azimuth_deg: float) -> np.ndarray:
    """9 x 9 float32 map from the ENZ tensor (rows of ENZ_ORDER) to the RTZ
    tensor (RTZ_ORDER): the outer product of the source basis (R = E sin az
    + N cos az, T = E cos az - N sin az) and the receiver basis (R = -E sin
    baz - N cos baz, T = -E cos baz + N sin baz), Z unchanged."""
    az = np.float32(np.deg2rad(azimuth_deg))
    baz = np.float32(np.deg2rad(back_azimuth_deg))
    sa, ca = np.sin(az, dtype=np.float32), np.cos(az, dtype=np.float32)
    sb, cb = np.sin(baz, dtype=np.float32), np.cos(baz, dtype=np.float32)
    one, zero = np.float32(1.0), np.float32(0.0)
    src = ((sa, ca, zero), (ca, -sa, zero), (zero, zero, one))
    rec = ((-sb, -cb, zero), (-cb, sb, zero), (zero, zero, one))
    m = np.zeros((9, 9), dtype=np.float32)
    # horizontal factors couple only horizontal components and Z only Z; a
    # Z factor (1) leaves the other factor unrounded
    linked = lambda i, a: (i < 2 and a < 2) or (i == 2 and a == 2)  # noqa: E731
    for i in range(3):
        for j in range(3):
            for a in range(3):
                for b in range(3):
                    if not (linked(i, a) and linked(j, b)):
                        continue
                    s, r = src[i][a], rec[j][b]
                    m[i * 3 + j, a * 3 + b] = r if i == 2 else (s if j == 2 else s * r)
    return m


class _Rotator:
    def __init__(self, ctx=None):
        import torch

        from .core import Context

        if not torch.cuda.is_available():
            raise RuntimeError("the GPU rotation needs a CUDA device")
        self.torch = torch
        self.ctx = ctx or Context(torch.cuda.current_device(), torch.cuda.current_stream().cuda_stream)

    def __call__(self, enz: np.ndarray, mats: np.ndarray) -> np.ndarray:
        """enz [P][9][npts] float32, mats [P][9][9] -> rtz [P][9][npts]."""
        import ctypes as C

        from ._lib import lib

        torch = self.torch
        enz = np.ascontiguousarray(enz, dtype=np.float32)
        npairs, _, npts = enz.shape
        d_in = torch.from_numpy(enz).cuda()
        d_m = torch.from_numpy(np.ascontiguousarray(mats, dtype=np.float32)).cuda()
        d_out = torch.empty_like(d_in)
        lib().fxc_rotate_enz_rtz(self.ctx.handle, C.c_void_p(d_in.data_ptr()), npairs, npts, npts,
                                 C.c_void_p(d_m.data_ptr()), C.c_void_p(d_out.data_ptr()))
        self.ctx.synchronize()
        return d_out.cpu().numpy()


_rotator = None


def _get_rotator(ctx=None) -> _Rotator:
    global _rotator
    if ctx is not None:
        return _Rotator(ctx)
    if _rotator is None:
        _rotator = _Rotator()
    return _rotator


def rotate_enz_to_rtz(enz_data: np.ndarray, azimuth_deg: float, back_azimuth_deg: float, *, ctx=None) -> np.ndarray:
    enz = np.asarray(enz_data, dtype=np.float32)
    if enz.ndim != 2 or enz.shape[0] != 9:
        raise ValueError(f"ENZ data must have shape (9, npts), got {enz.shape}")
    m = build_rotate_matrix(azimuth_deg, back_azimuth_deg)
    return _get_rotator(ctx)(enz[None], m[None])[0]


def _defined(v: float) -> bool:
    return math.isfinite(v) and abs(v - sacbin.NULL_VALUE) > 1.0e-3


def _lat_trig(lat_deg: float, lat_rad: float) -> tuple:
    if lat_deg == 90.0:
        return 0.0, 1.0, _FLT_MAX
    if lat_deg == -90.0:
        return 0.0, -1.0, -_FLT_MAX
    c, s = math.cos(lat_rad), math.sin(lat_rad)
    return c, s, s / c


def distkm_az_baz_rudoe(evlo: float, evla: float, stlo: float, stla: float) -> tuple:
    """(gcarc deg, azimuth deg, back azimuth deg, distance km) on the WGS84
    ellipsoid: geocentric direction cosines for the arc and the azimuths,
    Rudoe's series for the distance (the convention of
    fastxc/inventory/planner.py:833-968 and the xc stage's cal_dist.c)."""
    if evlo == stlo and evla == stla:
        return 0.0, 0.0, 0.0, 0.0
    d2r, r2d = math.pi / 180.0, 180.0 / math.pi
    radius = 6378.137
    flat = 1.0 / 298.257223563
    ec2 = 2.0 * flat - flat * flat
    om = 1.0 - ec2

    def cosines(lat, lon):
        lat_r = d2r * (lat if lat != 0.0 else 1.0e-10)
        lon_r = d2r * lon
        geoc = lat * d2r if lat in (90.0, -90.0) else math.atan(om * math.tan(lat_r))
        d, e = math.sin(lon_r), -math.cos(lon_r)
        f, c = -math.cos(geoc), math.sin(geoc)
        return lat_r, lon_r, (f * e, -f * d, c, d, e, f, -c * e, c * d)

    evla_r, evlo_r, (a, b, c, d, e, f, g, h) = cosines(evla, evlo)
    stla_r, stlo_r, (a1, b1, c1, d1, e1, f1, g1, h1) = cosines(stla, stlo)

    sc = a * a1 + b * b1 + c * c1
    sd = 0.5 * math.sqrt(((a - a1) ** 2 + (b - b1) ** 2 + (c - c1) ** 2) *
                         ((a + a1) ** 2 + (b + b1) ** 2 + (c + c1) ** 2))
    gcarc = math.atan2(sd, sc) * r2d
    if gcarc < 0.0:
        gcarc += 360.0

    def bearing(ss, cc):
        ang = math.atan2(ss, cc) * r2d
        if ang < 0.0 and abs(ang) < 1.0e-8:
            ang = 0.0
        return ang + 360.0 if ang < 0.0 else ang

    az = bearing((a1 - d) ** 2 + (b1 - e) ** 2 + c1 ** 2 - 2.0, (a1 - g) ** 2 + (b1 - h) ** 2 + (c1 - f) ** 2 - 2.0)
    baz = bearing((a - d1) ** 2 + (b - e1) ** 2 + c ** 2 - 2.0, (a - g1) ** 2 + (b - h1) ** 2 + (c - f1) ** 2 - 2.0)

    if stla_r > 0.0:
        p1, p2 = stlo_r, evlo_r
        ck, sk, tk = _lat_trig(evla, evla_r)
        ci, si, ti = _lat_trig(stla, stla_r)
    else:
        p1, p2 = evlo_r, stlo_r
        ck, sk, tk = _lat_trig(stla, stla_r)
        ci, si, ti = _lat_trig(evla, evla_r)
    ee = ec2 / om
    e1r = 1.0 + ee
    al = ti / (e1r * tk) + ec2 * math.sqrt((e1r + ti ** 2) / (e1r + tk ** 2))
    dl = p1 - p2
    a12 = math.atan2(math.sin(dl), (al - math.cos(dl)) * sk)
    ca12, sa12 = math.cos(a12), math.sin(a12)
    q1 = ee * ((ck * ca12) ** 2 + sk ** 2)
    q2 = q1 * q1
    q3 = q1 * q2
    c0 = 1.0 + 0.25 * q1 - (3.0 / 64.0) * q2 + (5.0 / 256.0) * q3
    c2 = -(1.0 / 8.0) * q1 + (13.0 / 32.0) * q2 - (15.0 / 1024.0) * q3
    c4 = -(1.0 / 256.0) * q2 + (3.0 / 1024.0) * q3
    v1 = radius / math.sqrt(1.0 - ec2 * sk ** 2)
    v2 = radius / math.sqrt(1.0 - ec2 * si ** 2)
    z1 = v1 * om * sk
    z2 = v2 * om * si
    x2 = v2 * ci * math.cos(dl)
    y2 = v2 * ci * math.sin(dl)
    q1p = q1 + 1.0
    sq = math.sqrt(q1p)
    u1 = math.atan2(tk, sq * ca12)
    u2 = math.atan2(v1 * sk + q1p * (z2 - z1), sq * (x2 * ca12 - y2 * sk * sa12))
    b0 = v1 * math.sqrt(1.0 + ee * (ck * ca12) ** 2) / q1p
    du = u2 - u1
    if abs(du) > math.pi:
        du = (math.pi * 2.0 - abs(du)) if du > 0.0 else (abs(du) - math.pi * 2.0)
    pdist = b0 * (c2 * (math.sin(2.0 * u2) - math.sin(2.0 * u1)) + c4 * (math.sin(4.0 * u2) - math.sin(4.0 * u1)))
    return gcarc, az, baz, abs(b0 * c0 * du + pdist)


def geometry_from_header(hd: sacbin.Header) -> tuple:
    ev = [hd.get_float(k) for k in ("evlo", "evla", "stlo", "stla")]
    if all(_defined(v) for v in ev):
        return distkm_az_baz_rudoe(*ev)
    gcarc, az, baz, dist = (hd.get_float(k) for k in ("gcarc", "az", "baz", "dist"))
    if _defined(az) and _defined(baz):
        return gcarc, az, baz, dist
    raise ValueError("Cannot determine azimuth/back-azimuth from SAC header")


def _rotated_base_header(template: sacbin.Header, geo: tuple) -> sacbin.Header:
    gcarc, az, baz, dist = geo
    h = template.copy()
    h.set_float("gcarc", float(gcarc))
    h.set_float("az", float(az))
    h.set_float("baz", float(baz))
    h.set_float("dist", float(dist))
    h.set_float("cmpaz", float(baz + 180.0 if baz - 180.0 < 0.0 else baz - 180.0))
    h.set_float("cmpinc", 90.0)
    return h


def _check_same_shape(names, headers) -> tuple:
    npts = headers[8].npts
    delta = headers[8].get_float("delta")
    for name, h in zip(names, headers):
        if h.npts != npts:
            raise ValueError(f"{name}: npts mismatch ({h.npts} vs {npts})")
        if not np.isclose(h.get_float("delta"), delta, rtol=0.0, atol=1.0e-7):
            raise ValueError(f"{name}: delta mismatch ({h.get_float('delta')} vs {delta})")
    return npts, delta


def rotate_sac_files(input_paths, output_paths, *, dry_run: bool = False, ctx=None) -> RotateResult:
    if len(input_paths) != 9 or len(output_paths) != 9:
        raise ValueError("rotate_sac_files expects exactly 9 input and 9 output paths")
    inputs = tuple(Path(p).expanduser().resolve() for p in input_paths)
    outputs = tuple(Path(p).expanduser().resolve() for p in output_paths)
    if dry_run:
        return RotateResult(Path("<direct>"), Path("<direct>"), outputs, 0)
    recs = [sacbin.read_file(p) for p in inputs]
    headers = [r[0] for r in recs]
    npts, _ = _check_same_shape(inputs, headers)
    geo = geometry_from_header(headers[8])
    enz = np.stack([r[1] for r in recs]).astype(np.float32, copy=False)
    rtz = _get_rotator(ctx)(enz[None], build_rotate_matrix(geo[1], geo[2])[None])[0]
    base = _rotated_base_header(headers[8], geo)
    for i, out in enumerate(outputs):
        h = base.copy()
        h.set_text("kcmpnm", SAC_COMPONENT_NAMES[i])
        sacbin.write_file(out, h, rtz[i])
    return RotateResult(Path("<direct>"), Path("<direct>"), outputs, npts)


def _read_list(path, expected: int = 9) -> list:
    path = Path(path).expanduser().resolve()
    rows = [Path(ln.strip()).expanduser().resolve() for ln in path.read_text().splitlines() if ln.strip()]
    if len(rows) != expected:
        raise ValueError(f"{path}: expected {expected} paths, got {len(rows)}")
    return rows


def rotate_from_lists(input_list, output_list, *, dry_run: bool = False, ctx=None) -> RotateResult:
    input_list = Path(input_list).expanduser().resolve()
    output_list = Path(output_list).expanduser().resolve()
    outputs = tuple(_read_list(output_list))
    if dry_run:
        return RotateResult(input_list, output_list, outputs, 0)
    r = rotate_sac_files(_read_list(input_list), outputs, ctx=ctx)
    return RotateResult(input_list, output_list, outputs, r.sample_count)


def discover_rotate_list_pairs(output_dir) -> list:
    root = Path(output_dir).expanduser().resolve() / "rotate_list"
    if not root.is_dir():
        return []
    return [(p, p.with_name("rtz_list.txt")) for p in sorted(root.glob("*/*/enz_list.txt"))
            if p.with_name("rtz_list.txt").is_file()]


def rotate_many_from_lists(list_pairs, *, max_workers: int = 1, dry_run: bool = False) -> list:
    tasks = [(Path(a).expanduser().resolve(), Path(b).expanduser().resolve()) for a, b in list_pairs]
    if not tasks:
        return []
    if max(1, int(max_workers)) == 1 or len(tasks) == 1:
        return [rotate_from_lists(a, b, dry_run=dry_run) for a, b in tasks]
    with concurrent.futures.ThreadPoolExecutor(max_workers=int(max_workers)) as pool:
        futs = [pool.submit(rotate_from_lists, a, b, dry_run=dry_run) for a, b in tasks]
        out = [f.result() for f in concurrent.futures.as_completed(futs)]
    return sorted(out, key=lambda r: str(r.input_list))


def _row_path_id(row: dict) -> str:
    pid = row.get("path_id", "").strip()
    if pid:
        return pid.zfill(8) if pid.isdigit() else pid
    try:
        return f"{int(row['src_id']) * 10000 + int(row['rec_id']):08d}"
    except (KeyError, ValueError):
        return ""


def _slot(src: str, rec: str) -> int:
    def rank(c: str) -> int:
        t = c.upper()[-1:] if c else ""
        return {"E": 0, "1": 0, "R": 0, "N": 1, "2": 1, "T": 1, "Z": 2, "3": 2}.get(t, 100)

    return rank(src) * 3 + rank(rec)


def _legacy_rtz_path(output_dir: Path, legacy: str, row: dict, tag: str) -> Path:
    pair = f"{row['src_network']}-{row['rec_network']}.{row['src_station']}-{row['rec_station']}"
    return output_dir / "stack" / legacy / pair / f"{pair}.{tag}.sac"


def _read_groups(index_path: Path) -> dict:
    groups: dict = {}
    with index_path.open("r", encoding="utf-8-sig", newline="") as fh:
        reader = csv.DictReader(fh, delimiter="\t")
        if reader.fieldnames is None:
            return groups
        need = {"source_key", "receiver_key", "record_path", "record_offset", "bytes", "src_component",
                "rec_component"}
        missing = need.difference(reader.fieldnames)
        if missing:
            raise ValueError(f"Sourcepack index missing fields {sorted(missing)}: {index_path}")
        for row in reader:
            groups.setdefault((_row_path_id(row), row["source_key"], row["receiver_key"]), []).append(row)
    return groups


def _rotated_row(template: dict, src_c: str, rec_c: str, pack_path: Path, offset: int, nbytes: int,
                 final_path: Path, hd: sacbin.Header, geo: tuple, storage_kind: str) -> dict:
    gcarc, az, baz, dist = geo
    row = {f: "" for f in SOURCEPACK_INDEX_HEADER}
    for key in ("path_id", "source_key", "receiver_key", "src_id", "rec_id", "src_network", "src_station",
                "src_location", "rec_network", "rec_station", "rec_location"):
        row[key] = template.get(key, "")
    row.update({
        "timestamp": "ROTATE",
        "path_id": _row_path_id(template),
        "component_slot": str(_slot(src_c, rec_c)),
        "src_component": src_c,
        "rec_component": rec_c,
        "npts": str(hd.npts),
        "dt": f"{hd.get_float('delta'):.9g}",
        "dist": f"{dist:.9g}",
        "az": f"{az:.9g}",
        "baz": f"{baz:.9g}",
        "record_path": pack_path.as_posix(),
        "record_offset": str(offset),
        "bytes": str(nbytes),
        "storage_kind": storage_kind,
        "final_pair_path": final_path.as_posix(),
    })
    return row


def rotate_sourcepack_stack(output_dir, method: str, *, dry_run: bool = False, ctx=None,
                            batch_pairs: int = 4096) -> list:
    """Rotate every complete nine-component pair of
    ``<output_dir>/stack/<method>_sourcepack/STACK`` into
    ``<output_dir>/stack/rtz_<method>_sourcepack/STACK`` (pack, index,
    ``_SUCCESS``); pairs missing a component are skipped and counted."""
    output_dir = Path(output_dir).expanduser().resolve()
    method = method.strip().lower()
    legacy = f"rtz_{method}"
    storage_kind = f"rtz_{method}_pack"
    index_path = output_dir / "stack" / f"{method}_sourcepack" / "STACK" / "sourcepack_index.tsv"
    if not index_path.is_file():
        raise FileNotFoundError(f"{method} sourcepack index not found: {index_path}")
    groups = sorted(_read_groups(index_path).items(), key=lambda kv: (_row_path_id(kv[1][0] if kv[1] else {}),
                                                                      kv[0][1], kv[0][2]))
    out_dir = output_dir / "stack" / f"rtz_{method}_sourcepack" / "STACK"
    pack_path = out_dir / f"rtz_{method}.pack"
    out_index = out_dir / "sourcepack_index.tsv"
    if dry_run:
        return [RotateResult(index_path, out_index,
                             tuple(_legacy_rtz_path(output_dir, legacy, rows[0], t) for t in RTZ_ORDER), 0)
                for _, rows in groups]

    tmp = out_dir.with_name(out_dir.name + ".tmp")
    if tmp.exists():
        shutil.rmtree(tmp)
    tmp.mkdir(parents=True, exist_ok=True)
    rot = _get_rotator(ctx)
    results: list = []
    skipped = 0
    handles: dict = {}

    def read(row: dict):
        rp = Path(row["record_path"]).expanduser()
        fh = handles.get(rp)
        if fh is None:
            fh = handles[rp] = rp.open("rb")
        return sacbin.read_record_from(fh, rp, int(row["record_offset"]), int(row["bytes"]))

    try:
        with (tmp / pack_path.name).open("wb") as pack, \
                (tmp / out_index.name).open("w", encoding="utf-8", newline="") as idx:
            writer = csv.DictWriter(idx, fieldnames=SOURCEPACK_INDEX_HEADER, delimiter="\t")
            writer.writeheader()
            pending = []  # (rows, template header, geometry, enz [9][npts])

            def flush():
                if not pending:
                    return
                enz = np.stack([p[3] for p in pending])
                mats = np.stack([build_rotate_matrix(p[2][1], p[2][2]) for p in pending])
                rtz = rot(enz, mats)
                for (rows, template, geo, _), out in zip(pending, rtz):
                    base = _rotated_base_header(template, geo)
                    paths = []
                    for i, tag in enumerate(RTZ_ORDER):
                        src_c, rec_c = tag.split("-")
                        h = base.copy()
                        h.set_text("kcmpnm", SAC_COMPONENT_NAMES[i])
                        off = pack.tell()
                        blob = sacbin.encode_record(h, out[i])
                        pack.write(blob)
                        row = _rotated_row(rows[0], src_c, rec_c, pack_path, off, len(blob),
                                           _legacy_rtz_path(output_dir, legacy, rows[0], tag), h, geo, storage_kind)
                        writer.writerow(row)
                        paths.append(Path(row["final_pair_path"]))
                    results.append(RotateResult(index_path, out_index, tuple(paths), template.npts))
                pending.clear()

            for _, rows in groups:
                by_cmp = {f"{r['src_component']}-{r['rec_component']}": r for r in rows}
                if any(t not in by_cmp for t in ENZ_ORDER):
                    skipped += 1
                    continue
                recs = [read(by_cmp[t]) for t in ENZ_ORDER]
                headers = [r[0] for r in recs]
                _check_same_shape([by_cmp[t]["record_path"] for t in ENZ_ORDER], headers)
                geo = geometry_from_header(headers[8])
                enz = np.stack([r[1] for r in recs]).astype(np.float32, copy=False)
                if pending and pending[0][3].shape[1] != enz.shape[1]:
                    flush()  # one trace length per GPU batch
                pending.append((rows, headers[8], geo, enz))
                if len(pending) >= batch_pairs:
                    flush()
            flush()
    finally:
        for fh in handles.values():
            fh.close()

    (tmp / "_SUCCESS").write_text(f"pairs\t{len(results)}\nskipped\t{skipped}\npack\t{pack_path}\n"
                                  f"index\t{out_index}\n", encoding="utf-8")
    if out_dir.exists():
        shutil.rmtree(out_dir)
    tmp.replace(out_dir)
    return results


def rotate_linearstack_sourcepack(output_dir, *, dry_run: bool = False, ctx=None) -> list:
    return rotate_sourcepack_stack(output_dir, "linearstack", dry_run=dry_run, ctx=ctx)
