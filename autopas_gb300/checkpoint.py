"""Particle checkpoints in md-flexible's rank-record layout (VTK UnstructuredGrid, ASCII), the same format as
include/autopas_gb300/Checkpoint.h: point data velocities, forces, typeIds, ids, then the positions
(examples/md-flexible/src/ParallelVtkWriter.cpp:55-200; read back as MDFlexConfig.cpp:91-180 does).  Numbers are
written with 17 significant digits, so a checkpoint restores the FP64 state exactly.
"""
from __future__ import annotations

import re

import numpy as np


def write_rank_record(filename, pos, vel, forces, type_ids, ids):
    pos, vel, forces = (np.asarray(a, np.float64).reshape(-1, 3) for a in (pos, vel, forces))
    n = len(pos)
    t = np.asarray(type_ids, np.int64).reshape(-1)
    i = np.asarray(ids, np.int64).reshape(-1)

    def vec3(name, a):
        rows = "\n".join(f"        {x!r} {y!r} {z!r}" for x, y, z in a.tolist())
        return (f'        <DataArray Name="{name}" NumberOfComponents="3" format="ascii" type="Float64">\n'
                f"{rows}\n        </DataArray>\n")

    def scal(name, a):
        rows = "\n".join(f"        {v}" for v in a.tolist())
        return (f'        <DataArray Name="{name}" NumberOfComponents="1" format="ascii" type="Int64">\n'
                f"{rows}\n        </DataArray>\n")

    with open(filename, "w") as f:
        f.write('<?xml version="1.0" encoding="UTF-8" standalone="no" ?>\n')
        f.write('<VTKFile byte_order="LittleEndian" type="UnstructuredGrid" version="0.1">\n')
        f.write("  <UnstructuredGrid>\n")
        f.write(f'    <Piece NumberOfCells="0" NumberOfPoints="{n}">\n')
        f.write("      <PointData>\n")
        f.write(vec3("velocities", vel))
        f.write(vec3("forces", forces))
        f.write(scal("typeIds", t))
        f.write(scal("ids", i))
        f.write("      </PointData>\n      <CellData/>\n      <Points>\n")
        f.write(vec3("positions", pos))
        f.write("      </Points>\n      <Cells>\n")
        f.write('        <DataArray Name="types" NumberOfComponents="0" format="ascii" type="Float32"/>\n')
        f.write("      </Cells>\n    </Piece>\n  </UnstructuredGrid>\n</VTKFile>\n")


def read_rank_record(filename):
    """Returns dict(pos, vel, forces, type_ids, ids) from a record written here or by md-flexible."""
    text = open(filename).read()
    n = int(re.search(r'NumberOfPoints="(\d+)"', text).group(1))

    def block(name, cols, dtype):
        m = re.search(r'Name="%s"[^\n]*\n(.*?)</DataArray>' % name, text, flags=re.S)
        vals = np.array(m.group(1).split(), dtype=dtype)
        return vals.reshape(n, cols) if cols > 1 else vals

    return {"vel": block("velocities", 3, np.float64), "forces": block("forces", 3, np.float64),
            "type_ids": block("typeIds", 1, np.int64), "ids": block("ids", 1, np.int64),
            "pos": block("positions", 3, np.float64)}
