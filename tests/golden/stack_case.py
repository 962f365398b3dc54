"""A small nine-component stacking case: two station pairs x the nine
E/N/Z component pairs, 5 daily NCFs of 201 lags each at 0.1 s, SAC headers
carrying the stations' coordinates (so that rotation finds the geometry);
components named E, N and Z, the names the rotation step matches.

tests/golden/make_stack_sample.py runs
this build's ncf_pws, ncf_tfpws and RTZ rotation on it (GPU) and commits the
outputs as tests/golden/stack_sample; tests/test_stack_reference_reader.py
regenerates the inputs here on the CPU to check those outputs.
"""

from __future__ import annotations

from pathlib import Path

import numpy as np

from fastxc_gb300 import formats
from fastxc_gb300.synthetic import ncf_traces

HERE = Path(__file__).resolve().parent
SAMPLE = HERE / "stack_sample"
NTS, NSAMPLES, DELTA, SEED = 5, 201, 0.1, 11
PWS_SUB, TFPWS_SUB, TFPWS_BAND = 3, 2, (0.2, 1.5)
COMPS = ("E", "N", "Z")
# path id -> (source station, source lat/lon, receiver station, receiver lat/lon)
PAIRS = {
    "3": ("SA", (35.0, -97.0), "RB", (36.2, -95.5)),
    "12": ("SC", (-10.0, 120.0), "RD", (-12.5, 118.0)),
}


def groups_order():
    """(path_id, src component, rec component) in the stacked index order
    (path ids as strings, then component slot)."""
    return [(p, a, b) for p in sorted(PAIRS) for a in COMPS for b in COMPS]


def traces() -> dict:
    """{(path_id, src component, rec component): float32 [NTS][NSAMPLES]}."""
    keys = groups_order()
    tr = ncf_traces(len(keys), NTS, NSAMPLES, delta=DELTA, seed=SEED)
    return {k: tr[i] for i, k in enumerate(keys)}


def write_inputs(root: Path) -> Path:
    """Two SourcePack index files (timestamps split between them) and the
    list file naming them; returns the list file."""
    root = Path(root)
    from fastxc_gb300.rotate import distkm_az_baz_rudoe

    tr = traces()
    rows = [[], []]
    for (pid, a, b), x in tr.items():
        s_sta, (s_la, s_lo), r_sta, (r_la, r_lo) = PAIRS[pid]
        _, az, baz, dist = distkm_az_baz_rudoe(s_lo, s_la, r_lo, r_la)
        for t in range(NTS):
            rows[t % 2].append(dict(
                timestamp=f"2021.{200 + t:03d}.0000", path_id=pid, component_slot=COMPS.index(a) * 3 + COMPS.index(b),
                source_key=f"XX.{s_sta}", receiver_key=f"XX.{r_sta}", src_id=pid, rec_id=str(int(pid) + 1),
                src_network="XX", src_station=s_sta, src_location="00", src_component=a,
                rec_network="XX", rec_station=r_sta, rec_location="00", rec_component=b,
                dist=f"{dist:.3f}", az=f"{az:.3f}", baz=f"{baz:.3f}", data=x[t], delta=DELTA,
                sac=dict(evla=s_la, evlo=s_lo, stla=r_la, stlo=r_lo),
                final_pair_path=f"stack/XX-XX.{s_sta}-{r_sta}.{a}-{b}.sac"))
    for part in (0, 1):
        rows[part].sort(key=lambda r: (r["path_id"], r["component_slot"], r["timestamp"]))
    idx = [formats.write_sourcepack(root / "in", f"part{i}", rows[i]) for i in (0, 1)]
    lst = root / "list.txt"
    lst.write_text("\n".join(str(p) for p in idx) + "\n")
    return lst
