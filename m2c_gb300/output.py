"""Solution snapshots in the layout the reference writes (Output.cpp:148-330,
520-560): one VTK XML RectilinearGrid file per snapshot whose points are the
cell centres, with the point fields density, velocity (3 components),
pressure, materialid and levelset0 (the names Output.cpp gives the vectors),
and a .pvd collection listing the snapshots with their times.  The data are
written inline as base64 little-endian float64 (readable by ParaView / VisIt;
the reference's PETSc viewer appends raw binary instead).
"""
import base64
import os
import struct

import numpy as np


def _b64(arr):
    raw = np.ascontiguousarray(arr, dtype="<f8").tobytes()
    return base64.b64encode(struct.pack("<Q", len(raw)) + raw).decode("ascii")


def write_vtr(path, cfg, V, ID, phi=None, time=None, fields=None):
    """Write one snapshot.  V: (N, 5) primitive state of the real cells
    (k-major, i fastest), ID: (N,), phi: (N,) or None.  fields: the point
    fields to write (names as below; the reference writes those switched On
    in Output, Output.cpp:268-330), or None for all."""
    nx, ny, nz = cfg.nx, cfg.ny, cfg.nz
    coords = []
    for n, lo, hi in ((nx, cfg.x0, cfg.xmax), (ny, cfg.y0, cfg.ymax), (nz, cfg.z0, cfg.zmax)):
        h = (hi - lo) / n
        coords.append(lo + 0.5 * h + np.arange(n) * h)      # MeshGenerator.cpp:166-171
    V = np.asarray(V, np.float64).reshape(-1, 5)
    want = None if fields is None else set(fields)
    fields = [("density", V[:, 0], 1), ("velocity", V[:, 1:4], 3), ("pressure", V[:, 4], 1),
              ("materialid", np.asarray(ID, np.float64), 1)]
    if phi is not None and cfg.n_levelsets > 0:
        fields.append(("levelset0", np.asarray(phi, np.float64), 1))
    if want is not None:
        fields = [f for f in fields if f[0] in want]
    ext = f"0 {nx - 1} 0 {ny - 1} 0 {nz - 1}"
    with open(path, "w") as f:
        f.write('<?xml version="1.0"?>\n')
        f.write('<VTKFile type="RectilinearGrid" version="1.0" byte_order="LittleEndian" header_type="UInt64">\n')
        f.write(f'  <RectilinearGrid WholeExtent="{ext}">\n')
        if time is not None:
            f.write('    <FieldData>\n')
            f.write(f'      <DataArray type="Float64" Name="TimeValue" NumberOfTuples="1" format="ascii">{time!r}'
                    '</DataArray>\n')
            f.write('    </FieldData>\n')
        f.write(f'    <Piece Extent="{ext}">\n')
        f.write('      <PointData Scalars="density" Vectors="velocity">\n')
        for name, data, ncomp in fields:
            f.write(f'        <DataArray type="Float64" Name="{name}" NumberOfComponents="{ncomp}" format="binary">')
            f.write(_b64(data))
            f.write('</DataArray>\n')
        f.write('      </PointData>\n')
        f.write('      <Coordinates>\n')
        for axis, c in zip("xyz", coords):
            f.write(f'        <DataArray type="Float64" Name="{axis}" format="binary">{_b64(c)}</DataArray>\n')
        f.write('      </Coordinates>\n')
        f.write('    </Piece>\n')
        f.write('  </RectilinearGrid>\n')
        f.write('</VTKFile>\n')


def write_pvd(path, entries):
    """The collection file: entries = [(time, snapshot file name relative to the .pvd), ...]."""
    with open(path, "w") as f:
        f.write('<?xml version="1.0"?>\n')
        f.write('<VTKFile type="Collection" version="0.1"\n')
        f.write('byte_order="LittleEndian">\n')
        f.write('  <Collection>\n')
        for t, name in entries:
            f.write('  <DataSet timestep="%e" file="%s"/>\n' % (t, name))
        f.write('  </Collection>\n')
        f.write('</VTKFile>\n')


class SolutionSeries:
    """Snapshots `<prefix><base>_NNNN.vtr` plus `<prefix><base>.pvd`, numbered
    like the reference's (Output.cpp:223-248)."""

    def __init__(self, prefix, base="solution"):
        self.prefix, self.base = prefix, base
        self.entries = []
        os.makedirs(prefix or ".", exist_ok=True)

    def write(self, cfg, V, ID, phi, time, fields=None):
        name = f"{self.base}_{len(self.entries):04d}.vtr"
        write_vtr(os.path.join(self.prefix, name), cfg, V, ID, phi, time, fields)
        self.entries.append((time, name))
        write_pvd(os.path.join(self.prefix, self.base + ".pvd"), self.entries)
        return name


def read_vtr(path):
    """The point fields of a snapshot written by write_vtr (for tests and tools)."""
    import re
    txt = open(path).read()
    out = {}
    for name, ncomp, data in re.findall(r'Name="(\w+)" NumberOfComponents="(\d)" format="binary">([^<]*)<', txt):
        raw = base64.b64decode(data)
        n = struct.unpack("<Q", raw[:8])[0]
        a = np.frombuffer(raw[8:8 + n], "<f8")
        out[name] = a.reshape(-1, int(ncomp)) if int(ncomp) > 1 else a
    return out
