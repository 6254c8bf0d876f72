"""History output: the reference's `.hst` files for the Burgers package.

The Burgers package registers one MassHistory sum per octant of the domain
(benchmarks/burgers/burgers_package.cpp:98-135, 406-439); the history output appends a
row of (time, dt, cycle, nbtotal, sums...) whenever the simulation time passes the next
output time (src/outputs/outputs.cpp:434-464, src/outputs/history.cpp:40-210). The sums
run on the device in one launch (`pgb_history_mass`); this module only formats rows, in
the reference's layout, so that `burgers_diff.py`-style comparisons of two files work.
"""
import ctypes

import numpy as np

from . import _native as nat
from .mesh import _ptr, _stream


def octant_regions(xmin, xmax):
    """The eight octants of the box [xmin, xmax] in the package's order (x1 side outermost,
    x3 side innermost), as (8, 6) rows of x1min, x1max, x2min, x2max, x3min, x3max."""
    mid = [0.5 * (xmin[d] + xmax[d]) for d in range(3)]
    out = []
    for s1 in range(2):
        for s2 in range(2):
            for s3 in range(2):
                row = []
                for d, side in enumerate((s1, s2, s3)):
                    row += [mid[d] if side else xmin[d], xmax[d] if side else mid[d]]
                out.append(row)
    return np.array(out, np.float64)


def mass_history(mesh, field, regions, mesh_volume, stream=None):
    """Per-region sums of q*q*vol/(mesh_volume + 1e-20) over every component (host array)."""
    r = np.ascontiguousarray(regions, np.float64).reshape(-1, 6)
    out = np.zeros(r.shape[0], np.float64)
    mesh._ensure()
    nat.check(nat.lib().pgb_history_mass(mesh.handle, _ptr(field), field.shape[1], r.ctypes.data_as(ctypes.c_void_p),
                                         r.shape[0], float(mesh_volume), out.ctypes.data_as(ctypes.c_void_p),
                                         _stream(stream)), "pgb_history_mass")
    return out


class HistoryFile:
    """Appends history rows in the reference's format: a two-line header on the first
    write, then per row time and dt in `data_format`, cycle and block count as %12d,
    and the sums in `data_format` (the reference prepends one blank to the format)."""

    def __init__(self, path, labels, data_format="%.14e"):
        self.path = path
        self.labels = list(labels)
        self.fmt = " " + data_format
        self.rows = 0

    def header(self):
        s = "#  History data\n"
        s += "# [1]=time    "
        s += " [2]=dt      "
        s += " [3]=cycle   "
        s += " [4]=nbtotal "
        for n, lab in enumerate(self.labels):
            s += " [%d]=%-8s" % (n + 5, lab)
        return s + "\n"

    def row(self, time, dt, cycle, nbtotal, values):
        s = self.fmt % time + self.fmt % dt + " %12d" % cycle + " %12d" % nbtotal
        for v in values:
            s += self.fmt % v
        return s + "\n"

    def write(self, time, dt, cycle, nbtotal, values):
        with open(self.path, "a" if self.rows else "w") as f:
            if self.rows == 0:
                f.write(self.header())
            f.write(self.row(time, dt, cycle, nbtotal, values))
        self.rows += 1


class BurgersHistory:
    """The Burgers package's history output: octant masses every `dt_out` of simulation
    time (and at cycle 0), written to `path`."""

    def __init__(self, path, xmin, xmax, dt_out, data_format="%.14e"):
        self.regions = octant_regions(xmin, xmax)
        self.volume = float(np.prod([xmax[d] - xmin[d] for d in range(3)]))
        self.dt_out = float(dt_out)
        self.next_time = 0.0
        self.file = HistoryFile(path, ["MS Mass %d" % i for i in range(8)], data_format)

    def maybe_write(self, mesh, field, dt_state, ncycle, stream=None):
        """dt_state: the driver's device array (dt, previous dt, time)."""
        import torch
        with torch.cuda.stream(stream):
            d = dt_state.cpu().numpy()
        dt, time = float(d[0]), float(d[2])
        if ncycle == 0 or time >= self.next_time:
            self.file.write(time, dt, ncycle, mesh.nblocks, mass_history(mesh, field, self.regions, self.volume,
                                                                          stream))
            self.next_time += self.dt_out
            return True
        return False
