"""On-disk formats of the reference for the fluid step's particle state.

* VTK XML PolyData state files, as BodyStatesRecordingToVtp writes them without the VTK
  library (src/shared/io_system/io_vtk.cpp:165-248, io_vtk.hpp:10-110): one file
  ``<BodyName>_<sequence>.vtp`` per body with the physical time as field data, the particle
  positions as points, a ``SortedParticle_ID`` array, then every variable added with
  ``addToWrite`` (u32 as Int32, scalars as Float32, vectors as 3-component Float32, dim x
  dim matrices as 9-component Float32 in column order), and one vertex per particle.
  The sequence is ``ite_`` + the zero-padded iteration, or the physical time in
  microseconds zero-padded to 10 digits (io_base.cpp:14-54).
* Restart files as RestartIO writes them (io_base.cpp:67-110, base_particles.cpp:166-182):
  ``Restart_<10-digit step>.xml`` with a ``restart_data`` root element carrying the
  ``restart_time`` attribute, one ``body`` element per real body (``name`` attribute), one
  ``particle`` child per particle whose attributes are the body's variables (vectors and
  matrices as comma-separated entries).  Values are written with 17 significant digits,
  so a restart continues bit for bit; the reference writes 15 and reads any precision.

The files are written from host copies of the device state (``SPHBody.download``) and
read back with ``SPHBody.upload``.
"""
from __future__ import annotations

import os
import xml.etree.ElementTree as ET
from typing import Dict, Iterable, List, Optional, Sequence, Tuple

import numpy as np


def pad(value, width: int = 10) -> str:
    """padValueWithZeros (io_base.h:72-77)."""
    return str(value).rjust(width, "0")


def vtp_sequence(iteration: Optional[int] = None, physical_time: Optional[float] = None) -> str:
    if iteration is not None:
        return "ite_" + pad(int(iteration))
    return pad(int(float(physical_time) * 1.0e6))


def _fixed9(values: np.ndarray) -> str:
    return " ".join(f"{v:.9f}" for v in np.asarray(values, dtype=np.float64).ravel())


def _upgrade3(a: np.ndarray) -> np.ndarray:
    a = np.asarray(a, dtype=np.float64)
    if a.ndim == 1:
        a = a[:, None]
    out = np.zeros((a.shape[0], 3))
    out[:, : a.shape[1]] = a
    return out


def write_vtp(path: str, name: str, position: np.ndarray, arrays: Sequence[Tuple[str, np.ndarray]],
              physical_time: Optional[float] = None) -> None:
    """One VTK XML PolyData file of n particles.  ``arrays`` holds (name, values) with
    values of shape (n,) u32 / float, (n, d) vectors or (n, d, d) matrices."""
    pos = _upgrade3(position)
    n = pos.shape[0]
    lines = ['<?xml version="1.0"?>',
             '<VTKFile type="PolyData" version="1.0" byte_order="LittleEndian">',
             ' <PolyData>']
    if physical_time is not None:
        lines += ["<FieldData>",
                  '<DataArray type="Float64"  Name="TimeValue" NumberOfTuples="1" format="ascii">',
                  f"{float(physical_time):.9f}", " </DataArray>", "</FieldData>"]
    lines += [f'  <Piece Name ="{name}" NumberOfPoints="{n}" NumberOfVerts="{n}">', "   <Points>",
              '    <DataArray Name="Position" type="Float32"  NumberOfComponents="3" format="ascii">',
              "    " + _fixed9(pos) + " ", "    </DataArray>", "   </Points>",
              '   <PointData  Vectors="vector">',
              '    <DataArray Name="SortedParticle_ID" type="Int32" format="ascii">',
              "    " + " ".join(str(i) for i in range(n)) + " ", "    </DataArray>"]
    for aname, values in arrays:
        v = np.asarray(values)
        if v.dtype.kind in "ui":
            lines += [f'    <DataArray Name="{aname}" type="Int32" format="ascii">',
                      "    " + " ".join(str(int(x)) for x in v.ravel()) + " "]
        elif v.ndim == 1:
            lines += [f'    <DataArray Name="{aname}" type="Float32" format="ascii">', "    " + _fixed9(v) + " "]
        elif v.ndim == 2:
            lines += [f'    <DataArray Name="{aname}" type="Float32"  NumberOfComponents="3" format="ascii">',
                      "    " + _fixed9(_upgrade3(v)) + " "]
        else:
            d = v.shape[1]
            m = np.zeros((v.shape[0], 3, 3))
            m[:, :d, :d] = v
            cols = np.transpose(m, (0, 2, 1))  # column by column, as Mat3d::col(k)
            lines += [f'    <DataArray Name="{aname}" type="Float32"  NumberOfComponents="9" format="ascii">',
                      "    " + _fixed9(cols) + " "]
        lines.append("    </DataArray>")
    lines += ["   </PointData>", "   <Verts>",
              '    <DataArray type="Int32"  Name="connectivity"  format="ascii">',
              "    " + " ".join(str(i) for i in range(n)) + " ", "    </DataArray>",
              '    <DataArray type="Int32"  Name="offsets"  format="ascii">',
              "    " + " ".join(str(i + 1) for i in range(n)) + " ", "    </DataArray>",
              "   </Verts>", "  </Piece>", " </PolyData>", "</VTKFile>"]
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def read_vtp(path: str) -> Dict[str, np.ndarray]:
    """Arrays of a state file by name ("Position" for the points, "TimeValue" if present);
    multi-component arrays come back as (n, components)."""
    root = ET.parse(path).getroot()
    out: Dict[str, np.ndarray] = {}
    for da in root.iter("DataArray"):
        nm = da.get("Name")
        txt = (da.text or "").split()
        kind = np.int64 if da.get("type") == "Int32" else np.float64
        a = np.array([kind(x) if kind is np.int64 else float(x) for x in txt])
        nc = int(da.get("NumberOfComponents", "1"))
        out[nm] = a.reshape(-1, nc) if nc > 1 else a
    return out


class BodyStatesRecordingToVtp:
    """BodyStatesRecordingToVtp(bodies) with addToWrite<T>(body, name) and writeToFile."""

    def __init__(self, bodies, output_folder: str = "output"):
        self.bodies = list(bodies) if isinstance(bodies, (list, tuple)) else list(bodies.bodies)
        self.folder = output_folder
        self.to_write: Dict[int, List[str]] = {}

    def addToWrite(self, body, name: str) -> None:
        self.to_write.setdefault(id(body), []).append(name)

    def writeToFile(self, iteration: Optional[int] = None, physical_time: float = 0.0) -> List[str]:
        os.makedirs(self.folder, exist_ok=True)
        seq = vtp_sequence(iteration, physical_time)
        paths = []
        for b in self.bodies:
            if getattr(b, "handle", None) is None or b.n == 0:
                continue
            arrays = []
            for nm in self.to_write.get(id(b), []):
                v = b.download(nm)
                if v.ndim == 2 and v.shape[1] == b.dim * b.dim and nm == "LinearCorrectionMatrix":
                    v = v.reshape(-1, b.dim, b.dim)
                arrays.append((nm, v))
            path = os.path.join(self.folder, f"{b.name}_{seq}.vtp")
            write_vtp(path, b.name, b.download("Position"), arrays, physical_time)
            paths.append(path)
        return paths


def _fmt17(v) -> str:
    a = np.asarray(v, dtype=np.float64).ravel()
    return ", ".join(f"{x:.17g}" for x in a)


def write_restart(path: str, physical_time: float, bodies: Sequence[Tuple[str, Dict[str, np.ndarray]]]) -> None:
    """Restart file of (body name, {variable: values}) in the RestartIO layout."""
    root = ET.Element("restart_data", {"restart_time": f"{float(physical_time):.17g}"})
    for bname, variables in bodies:
        be = ET.SubElement(root, "body", {"name": bname})
        n = min((len(v) for v in variables.values()), default=0)
        for i in range(n):
            ET.SubElement(be, "particle", {nm: _fmt17(v[i]) for nm, v in variables.items()})
    ET.indent(root, space="    ")
    ET.ElementTree(root).write(path, encoding="unicode", xml_declaration=False)


def read_restart(path: str) -> Tuple[float, Dict[str, Dict[str, np.ndarray]]]:
    """(restart time, {body name: {variable: (n,) or (n, components)}})."""
    root = ET.parse(path).getroot()
    t = float(root.get("restart_time"))
    out: Dict[str, Dict[str, np.ndarray]] = {}
    for be in root.findall("body"):
        parts = be.findall("particle")
        names = list(parts[0].attrib) if parts else []
        vars_: Dict[str, np.ndarray] = {}
        for nm in names:
            rows = [[float(x) for x in p.get(nm).split(",")] for p in parts]
            a = np.array(rows)
            vars_[nm] = a[:, 0] if a.shape[1] == 1 else a
        out[be.get("name")] = vars_
    return t, out


class RestartIO:
    """RestartIO(bodies): writeToFile(step, time) and readRestartFiles(step) for the
    variables the fluid step evolves (and the walls' geometry)."""

    FLUID = ("Position", "Velocity", "Force", "ForcePrior", "Density", "Pressure", "DensityChangeRate", "Mass",
             "VolumetricMeasure")
    SOLID = ("Position", "NormalDirection", "Mass", "VolumetricMeasure", "Density")

    def __init__(self, bodies, restart_folder: str = "restart"):
        self.bodies = list(bodies) if isinstance(bodies, (list, tuple)) else list(bodies.bodies)
        self.folder = restart_folder

    def _variables(self, b) -> Iterable[str]:
        names = self.FLUID if b.material is not None and hasattr(b.material, "c0") else self.SOLID
        return [nm for nm in names if _registered(b, nm)]

    def path(self, step: int) -> str:
        return os.path.join(self.folder, f"Restart_{pad(int(step))}.xml")

    def writeToFile(self, step: int, physical_time: float) -> str:
        os.makedirs(self.folder, exist_ok=True)
        bodies = [(b.name, {nm: b.download(nm) for nm in self._variables(b)}) for b in self.bodies
                  if getattr(b, "handle", None) is not None and b.n > 0 and hasattr(b, "mesh")]
        p = self.path(step)
        write_restart(p, physical_time, bodies)
        return p

    def readRestartFiles(self, step: int) -> float:
        """Loads every body found in the file (same particle counts) and returns the
        restart time; cell lists and relations must be rebuilt afterwards."""
        t, data = read_restart(self.path(step))
        for b in self.bodies:
            if b.name in data:
                for nm, v in data[b.name].items():
                    if len(v) != b.n:
                        raise ValueError(f"restart body {b.name}: {len(v)} particles for {b.n}")
                    b.upload(nm, v)
        return t


def _registered(body, name: str) -> bool:
    import ctypes as C
    from . import native as N
    ptr = C.c_void_p()
    return N._lib is not None and N.load().sphx_body_device_ptr(body.handle, name.encode(), C.byref(ptr), None,
                                                                 None) == 0
