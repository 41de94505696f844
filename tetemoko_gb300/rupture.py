"""Rupture metrics at fault stations: how the mixed form's rupture differs from
the FP64 form's.

From the fault-station records (tetemoko_gb300.stations, the values the
reference writes in its station files, srcLinElast/AMRLevelLinElast.cpp:1758-1869):
  * rupture-front arrival time: the first crossing of the slip-rate threshold
    (the deck's rupture velocity threshold, 1e-3 m/s), linear in time between
    records;
  * final slip: the total slip of the last record;
  * peak slip rate: the largest slip rate over the records;
and from the final states, the largest particle-velocity difference in the
volume relative to the largest particle velocity of the reference run.
"""
from __future__ import annotations

import numpy as np

from . import _capi as A

# boundary-data components (ibcLinElast/RSINDEX.H; SWSETBND, ibcLinElast/SWIBCF.ChF:32-72)
SLIP_RATE = {A.TMK_FAULT_RS: 2, A.TMK_FAULT_SW: 4}
SLIP_TOTAL = {A.TMK_FAULT_RS: 8, A.TMK_FAULT_SW: 7}
VELOCITY_COMPS = [0, 1, 2, 11, 12, 13]


def arrival_times(ts: np.ndarray, V: np.ndarray, threshold: float) -> np.ndarray:
    """First crossing of `threshold` by each column of the slip-rate history V
    (records x stations), linear in time between records; NaN if none."""
    out = []
    for k in range(V.shape[1]):
        v = V[:, k]
        idx = np.nonzero(v > threshold)[0]
        if len(idx) == 0:
            out.append(np.nan)
            continue
        n = idx[0]
        if n == 0:
            out.append(ts[0])
            continue
        a = (threshold - v[n - 1]) / (v[n] - v[n - 1])
        out.append(ts[n - 1] + a * (ts[n] - ts[n - 1]))
    return np.array(out)


def station_metrics(records: dict, fault_law: int, threshold: float) -> dict:
    """Arrival time, final slip and peak slip rate per fault station from the
    records of tetemoko_gb300.stations.Stations.read()."""
    V = records["fault"][:, :, SLIP_RATE[fault_law]]
    slip = records["fault"][-1, :, SLIP_TOTAL[fault_law]]
    return {"arrival": arrival_times(records["time"], V, threshold), "final_slip": slip.copy(),
            "peak_slip_rate": V.max(axis=0)}


def compare(test: dict, ref: dict) -> dict:
    """Largest relative differences of station_metrics `test` against `ref`
    (stations where the reference front never arrived are left out)."""
    ok = np.isfinite(ref["arrival"])
    out = {"stations": int(len(ok)), "stations_ruptured": int(ok.sum())}
    if not ok.any():
        out.update(arrival=None, final_slip=None, peak_slip_rate=None)
        return out
    ta, ra = test["arrival"][ok], ref["arrival"][ok]
    out["arrival"] = float(np.max(np.abs(ta - ra) / ra)) if np.all(np.isfinite(ta)) else float("inf")
    out["final_slip"] = float(np.max(np.abs(test["final_slip"][ok] - ref["final_slip"][ok]) /
                                     np.abs(ref["final_slip"][ok])))
    out["peak_slip_rate"] = float(np.max(np.abs(test["peak_slip_rate"][ok] - ref["peak_slip_rate"][ok]) /
                                         ref["peak_slip_rate"][ok]))
    return out


def velocity_error(U_test: np.ndarray, U_ref: np.ndarray, ghost: int = A.TMK_NGHOST) -> float:
    """Largest particle-velocity difference over the valid cells of two state
    FABs (22, ny + 2g, nx + 2g), relative to the reference's largest."""
    vs = (VELOCITY_COMPS, slice(ghost, -ghost), slice(ghost, -ghost))
    return float(np.abs(U_test[vs] - U_ref[vs]).max() / np.abs(U_ref[vs]).max())
