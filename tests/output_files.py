"""Readers of the .vtk and PETSc binary files the drop-in driver writes (tests only)."""
import numpy as np


def read_ptc(path: str) -> np.ndarray:
    """A vector written by petsc::write: class id 1211214 and length (big-endian int32),
    then big-endian doubles."""
    raw = open(path, "rb").read()
    head = np.frombuffer(raw[:8], dtype=">i4")
    assert head[0] == 1211214
    return np.frombuffer(raw[8:8 + 8 * int(head[1])], dtype=">f8").astype(np.float64)


def read_vtk(path: str) -> dict:
    """Points, cells, cell types and the named cell-data sections of a vtk.cxx file."""
    lines = open(path).read().split("\n")
    out = dict(scalars={})
    k = 0
    while k < len(lines):
        w = lines[k].split()
        if not w:
            k += 1
        elif w[0] == "POINTS":
            n = int(w[1])
            out["points"] = np.array([[float(x) for x in lines[k + 1 + i].split()] for i in range(n)])
            k += n + 1
        elif w[0] == "CELLS":
            n = int(w[1])
            out["cells"] = [[int(x) for x in lines[k + 1 + i].split()][1:] for i in range(n)]
            k += n + 1
        elif w[0] == "CELL_TYPES":
            n = int(w[1])
            out["types"] = [int(lines[k + 1 + i]) for i in range(n)]
            k += n + 1
        elif w[0] == "CELL_DATA":
            out["num_cells"] = int(w[1])
            k += 1
        elif w[0] == "SCALARS":
            n = out["num_cells"]
            out["scalars"][w[1]] = np.array([float(lines[k + 2 + i]) for i in range(n)])
            k += n + 2
        else:
            k += 1
    return out
