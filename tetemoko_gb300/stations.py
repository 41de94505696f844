"""Fault and body stations recorded on the device (AMRLevelLinElast's
writeStationLevel, srcLinElast/AMRLevelLinElast.cpp:1758-1869) and the
reference's station files.

A `Stations` object belongs to one level: each record (made by `record`, or
after every step once `attach`ed) interpolates the level's fault data and
state at the stations on the device; `read` copies the records out, and
`write_files` appends them to the files the reference writes
(AMRLevelLinElast::define, :282-370): per station and level a text header

    #number of values = N
    #size of real = 8
    #time<TAB>name...<TAB>level<TAB>procID

followed by records of N + 3 native doubles (time, values, level, procID).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _capi as A
from .level import _stream_ptr

# the names the reference writes in the headers (RSIBC::bdryNames,
# ibcLinElast/RSIBC.cpp:380-396; SWIBC::bdryNames, ibcLinElast/SWIBC.H:129-141;
# LinElastPhysics::stateNames, srcLinElast/LinElastPhysics.cpp:80-110)
RS_NAMES = ["Vx", "Vz", "V", "sxy", "syz", "syy", "slip x", "slip z", "slip total", "rupture time", "psi"]
SW_NAMES = ["Vx", "Vz", "sxy", "syz", "V", "slip_x", "slip_z", "slip_total", "rupture"]
STATE_NAMES = [f"{n}^{s}" for s in (1, 2) for n in ("v_x", "v_y", "v_z", "sig_xx", "sig_yy", "sig_zz", "sig_xy",
                                                     "sig_xz", "sig_yz", "lambda", "gamma")]


class Stations:
    """Stations of one level: fault stations at x along the fault, body
    stations at (x, y); `center` is the deck's domain centre offset."""

    def __init__(self, level, fault_x=(), body_xy=(), center=(0.0, 0.0), capacity: int = 4096):
        self.level = level
        self.lib = level.lib
        self.fault_x = [float(x) for x in fault_x]
        self.body_xy = [(float(x), float(y)) for x, y in body_xy]
        self.center = (float(center[0]), float(center[1]))
        self.nb = level.ctx.sc.nbdry
        nf, nbod = len(self.fault_x), len(self.body_xy)
        xf = (C.c_double * max(1, nf))(*self.fault_x)
        xb = (C.c_double * max(1, nbod))(*[p[0] for p in self.body_xy])
        yb = (C.c_double * max(1, nbod))(*[p[1] for p in self.body_xy])
        ce = (C.c_double * 2)(*self.center)
        h = C.c_void_p()
        self.h = None
        A.check(self.lib.tmk_stations_create(level.h, nf, xf, nbod, xb, yb, ce, capacity, C.byref(h)),
                "tmk_stations_create")
        self.h = h
        n = C.c_int(0)
        pres = (C.c_int * (nf + nbod))()
        A.check(self.lib.tmk_stations_layout(self.h, C.byref(n), pres), "tmk_stations_layout")
        self.stride = n.value
        self.present = [bool(v) for v in pres]
        self.capacity = capacity

    def record(self, time: float, stream=None):
        A.check(self.lib.tmk_stations_record(self.h, time, _stream_ptr(stream)), "tmk_stations_record")

    def attach(self):
        """Record after every step of the level (postTimeStep's order)."""
        A.check(self.lib.tmk_level_attach_stations(self.level.h, self.h), "tmk_level_attach_stations")

    def detach(self):
        A.check(self.lib.tmk_level_attach_stations(self.level.h, None), "tmk_level_attach_stations")

    def read(self):
        """Records since the last read: dict(time (n,), fault (n, nfault, nb),
        body (n, nbody, 22), dropped)."""
        buf = np.empty((self.capacity, self.stride))
        n = C.c_int(0)
        dropped = C.c_longlong(0)
        A.check(self.lib.tmk_stations_read(self.h, buf.ctypes.data_as(C.POINTER(C.c_double)), self.capacity,
                                           C.byref(n), C.byref(dropped)), "tmk_stations_read")
        r = buf[:n.value]
        nf = len(self.fault_x)
        nrec = r.shape[0]
        fault = r[:, 1:1 + nf * self.nb].reshape(nrec, nf, self.nb)
        body = r[:, 1 + nf * self.nb:].reshape(nrec, len(self.body_xy), 22)
        return {"time": r[:, 0].copy(), "fault": fault.copy(), "body": body.copy(), "dropped": dropped.value}

    # ---------------------------------------------------------------- files
    def file_names(self, prefix: str, level_index: int):
        """The reference's names: <prefix>Fx%5.4fz%5.4f.L%d.dat and
        <prefix>Bx%5.4fy%5.4fz%5.4f.L%d.dat (z = 0 in 2-D)."""
        f = [f"{prefix}Fx{x:5.4f}z{0.0:5.4f}.L{level_index}.dat" for x in self.fault_x]
        b = [f"{prefix}Bx{x:5.4f}y{y:5.4f}z{0.0:5.4f}.L{level_index}.dat" for x, y in self.body_xy]
        return f, b

    def write_files(self, prefix: str, level_index: int, records: dict, create: bool = False):
        """Append `records` (from read) to the station files; create=True
        starts them with the header first."""
        fnames, bnames = self.file_names(prefix, level_index)
        law = self.level.ctx.sc.scheme.fault_law
        bnames_ = RS_NAMES if law == A.TMK_FAULT_RS else SW_NAMES
        nf = len(self.fault_x)
        for k, name in enumerate(fnames + bnames):
            fault = k < nf
            names = bnames_ if fault else STATE_NAMES
            if create:
                with open(name, "w") as fh:
                    fh.write(f"#number of values = {len(names)}\n#size of real = 8\n#time")
                    fh.write("".join(f"\t{n}" for n in names))
                    fh.write("\tlevel\tprocID\n")
            if not self.present[k]:
                continue
            vals = records["fault"][:, k] if fault else records["body"][:, k - nf]
            n = len(records["time"])
            rows = np.empty((n, vals.shape[1] + 3))
            rows[:, 0] = records["time"]
            rows[:, 1:-2] = vals
            rows[:, -2] = level_index
            rows[:, -1] = 0.0
            with open(name, "ab") as fh:
                fh.write(rows.astype(np.float64).tobytes())

    def close(self):
        if self.h:
            self.lib.tmk_stations_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def read_station_file(name: str):
    """Parse a station file: (column names, records (n, ncols))."""
    with open(name, "rb") as fh:
        data = fh.read()
    lines = data.split(b"\n", 3)
    nvals = int(lines[0].split(b"=")[1])
    cols = lines[2].decode().lstrip("#").split("\t")
    body = lines[3] if len(lines) > 3 else b""
    rec = np.frombuffer(body, dtype=np.float64).reshape(-1, nvals + 3)
    return cols, rec
