"""Readers and writers for the reference's input files.

  lattice file   9 numbers; row i of the file is a_i
                 (Crystal_Lattice ctor reads bravais_lattice(j, i), bse.version13.cpp:94-97)
  atoms file     3 numbers per atom (bse.version13.cpp:99-102)
  *_hr.dat       Wannier90 format: header, nw, nR, nR weights, nw*nw*nR lines
                 "R1 R2 R3 l m Re Im" (crystal R); for collinear spin the file holds two
                 complete blocks, up then down (Hamiltonian_TB ctor, bse.version13.cpp:485-580)
  *_centres.xyz  count line, comment line, nw lines "X x y z", then the atoms
                 (repeated per spin channel, bse.version13.cpp:608-634)
  k list         3 numbers per line, crystal or cartesian (bse.version13.cpp:186-203)
  spectrum       output of pull_macroscopic_bse_dielectric_function (3644-3656): a header line, then
                 per frequency "(w,0) (eps_xx) (w,0) (eps_yy) (w,0) (eps_zz) Im(eps_avg)/3" with
                 complex numbers printed as "(re,im)"; only xx is computed, so yy = zz = (0,0) and the
                 last column is Im(eps_xx)/3 (quirk Q16)
  *.xsf          real-space Wannier functions on a supercell grid (Real_space_wannier ctor,
                 bse.version13.cpp:1081-1212): read_xsf_datagrid / read_wannier_xsf, write_xsf_datagrid

The reader keeps the reference's semantics: the R vectors of a block are the ones given
on the first line of each group of nw*nw lines, converted crystal->cartesian with the
lattice; weights are multiplied into H(k) by Hamiltonian_TB::FFT (quirk Q1 -- the
synthetic models write weight 1, so the Wannier90 divide-vs-multiply question is moot).
"""
from __future__ import annotations

import datetime
import os
from typing import Optional

import numpy as np

from .model import TBModel


def write_lattice(path, lattice: np.ndarray):
    with open(path, "w") as f:
        for i in range(3):
            f.write(" ".join(f"{x:.16e}" for x in lattice[:, i]) + "\n")


def read_lattice(path) -> np.ndarray:
    v = np.loadtxt(path).reshape(-1)[:9]
    lat = np.zeros((3, 3))
    for i in range(3):
        for j in range(3):
            lat[j, i] = v[3 * i + j]
    return lat


def write_atoms(path, atoms: np.ndarray):
    with open(path, "w") as f:
        for a in np.atleast_2d(atoms):
            f.write(" ".join(f"{x:.16e}" for x in a) + "\n")


def read_atoms(path, n_atoms: int) -> np.ndarray:
    return np.loadtxt(path).reshape(-1)[:3 * n_atoms].reshape(n_atoms, 3)


def write_hr(path, model: TBModel):
    nw, nr = model.nw, model.n_r
    with open(path, "w") as f:
        for s in range(model.n_spin):
            f.write(f"written on {datetime.date(2026, 1, 1).isoformat()} (synthetic model {model.name}, spin {s})\n")
            f.write(f"{nw:12d}\n{nr:12d}\n")
            for i in range(0, nr, 15):
                f.write("".join(f"{int(w):5d}" for w in model.weights[i:i + 15]) + "\n")
            for ir in range(nr):
                R = model.r_cryst[ir]
                for m in range(nw):
                    for l in range(nw):
                        h = model.h_r[s, ir, l, m]
                        f.write(f"{R[0]:5d}{R[1]:5d}{R[2]:5d}{l + 1:5d}{m + 1:5d} "
                                f"{h.real: .16e} {h.imag: .16e}\n")


def read_hr(path, nw: int, n_r: int, n_spin: int = 1):
    """Parse a (one- or two-block) hr.dat.  Returns (r_cryst (nR,3) int, weights (nR,),
    h_r (n_spin,nR,nw,nw)) and raises ValueError on a header mismatch (the reference
    prints "ERROR!!!!!!!" and continues, bse.version13.cpp:499-501)."""
    with open(path) as f:
        lines = f.read().split("\n")
    pos = 0
    h_r = np.zeros((n_spin, n_r, nw, nw), np.complex128)
    r_cryst = np.zeros((n_r, 3), np.int64)
    weights = np.zeros(n_r)
    for s in range(n_spin):
        while pos < len(lines) and not lines[pos].strip():
            pos += 1
        pos += 1                                 # header / date line
        toks = []
        while len(toks) < 2:
            toks += lines[pos].split()
            pos += 1
        nw_f, nr_f = int(toks[0]), int(toks[1])
        if nw_f != nw or nr_f != n_r:
            raise ValueError(f"hr.dat header mismatch: file has nw={nw_f} nR={nr_f}, expected {nw} {n_r}")
        w = []
        while len(w) < n_r:
            w += [float(x) for x in lines[pos].split()]
            pos += 1
        weights[:] = w[:n_r]
        total = nw * nw * n_r
        for cnt in range(total):
            t = lines[pos].split()
            pos += 1
            R = [int(float(x)) for x in t[:3]]
            l, m = int(t[3]), int(t[4])
            ir = cnt // (nw * nw)
            if cnt % (nw * nw) == 0:
                r_cryst[ir] = R
            h_r[s, ir, l - 1, m - 1] = float(t[5]) + 1j * float(t[6])
    return r_cryst, weights, h_r


def write_centres(path, model: TBModel, atoms: Optional[np.ndarray] = None):
    atoms = np.zeros((0, 3)) if atoms is None else np.atleast_2d(atoms)
    with open(path, "w") as f:
        for s in range(model.n_spin):
            f.write(f"{model.nw + len(atoms):6d}\n")
            f.write(f" Wannier centres, synthetic model {model.name}, spin {s}\n")
            for c in model.centres[s]:
                f.write("X " + " ".join(f"{x: .16e}" for x in c) + "\n")
            for a in atoms:
                f.write("A " + " ".join(f"{x: .16e}" for x in a) + "\n")


def read_centres(path, nw: int, n_atoms: int, n_spin: int = 1) -> np.ndarray:
    with open(path) as f:
        lines = [ln for ln in f.read().split("\n")]
    pos = 0
    out = np.zeros((n_spin, nw, 3))
    for s in range(n_spin):
        while pos < len(lines) and not lines[pos].strip():
            pos += 1
        pos += 2                                   # count line, comment line
        for i in range(nw):
            t = lines[pos].split()
            pos += 1
            out[s, i] = [float(x) for x in t[1:4]]
        pos += n_atoms
    return out


def write_klist(path, k: np.ndarray):
    np.savetxt(path, np.atleast_2d(k), fmt="%.16e")


def read_klist(path, n_k: int, shift=(0.0, 0.0, 0.0)) -> np.ndarray:
    k = np.loadtxt(path).reshape(-1, 3)[:n_k]
    return k + np.asarray(shift)[None, :]


def write_model_files(model: TBModel, directory, seedname: str, atoms=None):
    """Write lattice, atoms, hr.dat and centres.xyz for a model; returns the paths."""
    os.makedirs(directory, exist_ok=True)
    atoms = model.centres[0] if atoms is None else atoms
    paths = {
        "lattice": os.path.join(directory, f"bravais.lattice_{seedname}.data"),
        "atoms": os.path.join(directory, f"atoms_{seedname}.data"),
        "hr": os.path.join(directory, f"{seedname}_hr.dat"),
        "centres": os.path.join(directory, f"{seedname}_centres.xyz"),
    }
    write_lattice(paths["lattice"], model.lattice)
    write_atoms(paths["atoms"], atoms)
    write_hr(paths["hr"], model)
    write_centres(paths["centres"], model, atoms)
    return paths


def read_model_files(paths, nw: int, n_r: int, n_atoms: int, n_spin: int = 1,
                     dim: int = 3, name: str = "model") -> TBModel:
    lat = read_lattice(paths["lattice"])
    r_cryst, weights, h_r = read_hr(paths["hr"], nw, n_r, n_spin)
    centres = read_centres(paths["centres"], nw, n_atoms, n_spin)
    return TBModel(lattice=lat, r_cryst=r_cryst, weights=weights, h_r=h_r,
                   centres=centres, dim=dim, name=name)


def _cx(z: complex) -> str:
    return f"({z.real:.10g},{z.imag:.10g})"


def write_spectrum(path, omega, eps2, eps1):
    """The reference's dielectric-function file for eps_xx = eps1 + i eps2 (3644-3656)."""
    with open(path, "w") as fh:
        fh.write("### omega xx xy xz yx yy yz zx zy zz\n")
        for w, e2, e1 in zip(np.asarray(omega, float), np.asarray(eps2, float), np.asarray(eps1, float)):
            wc = _cx(complex(w, 0.0))
            fh.write(f"{wc} {_cx(complex(e1, e2))} {wc} (0,0) {wc} (0,0) {e2 / 3:.10g}\n")


def read_spectrum(path):
    """(omega, eps_xx) from a dielectric-function file in the reference's layout."""
    om, eps = [], []
    with open(path) as fh:
        for line in fh:
            if line.startswith("#") or not line.strip():
                continue
            f = line.split()
            w = complex(*map(float, f[0].strip("()").split(",")))
            e = complex(*map(float, f[1].strip("()").split(",")))
            om.append(w.real)
            eps.append(e)
    return np.asarray(om), np.asarray(eps)


def read_band_path(path, n_segments: int, crystal: bool = False, reciprocal=None):
    """Segments of a band-structure path, the file of Hamiltonian_TB::pull_bands
    (bse.version13.cpp:823-875): per segment "kx ky kz  kx ky kz  n" (start, end, points).
    crystal: coordinates in units of the reciprocal vectors (columns of `reciprocal`), converted
    to cartesian as 841-851 do.  Returns [(k_start, k_end, n), ...] in cartesian coordinates."""
    vals = np.loadtxt(path).reshape(-1, 7)[:n_segments]
    segs = []
    for row in vals:
        a, b, n = row[:3].copy(), row[3:6].copy(), int(row[6])
        if crystal:
            a, b = np.asarray(reciprocal) @ a, np.asarray(reciprocal) @ b
        segs.append((a, b, n))
    return segs


def band_path_points(segments) -> np.ndarray:
    """k points of the path: n points per segment from start to end inclusive (853-857)."""
    pts = []
    for a, b, n in segments:
        for j in range(n):
            t = j / (n - 1) if n > 1 else 0.0
            pts.append(a * (1.0 - t) + b * t)
    return np.asarray(pts).reshape(-1, 3)


def write_bands(path, e_v, e_c, n_spin: int):
    """The bands file of pull_bands (858-864): per k, for each spin row the selected valence
    bands (top-down from E_F) then the conduction bands (bottom-up, with the scissor)."""
    with open(path, "w") as fh:
        for k in range(e_v.shape[1]):
            row = []
            for s in range(n_spin):
                row += [f"{x:.10g}" for x in e_v[s, k]] + [f"{x:.10g}" for x in e_c[s, k]]
            fh.write(" ".join(row) + " \n")


# ------------------------------------------------------------------------------------------
# Real-space Wannier functions on an XSF data grid (Real_space_wannier ctor, bse.version13.cpp:
# 1081-1212).  File names: seedname + "_00001.xsf" (function w + 1, five digits); with spinor
# functions seedname + "up_00001.xsf" / "down_00001.xsf" (1108-1117).  The reference skips the
# first 22 lines of a file, then reads the grid dimensions, the origin, the three spanning vectors
# of the (super)cell grid and the values, x fastest over the whole supercell grid (1121-1139).
# The reader here finds the grid by its BEGIN_DATAGRID_3D keyword instead of a fixed line count
# (the count depends on the number of atoms in the header: quirk Q31); the writer emits exactly 22
# header lines before the dimensions, so the reference reads its files as they are.
# ------------------------------------------------------------------------------------------
def xsf_name(seedname: str, w: int, spinor: bool = False, spin: int = 0) -> str:
    """The reference's file name of Wannier function w (0-based) of spin channel `spin`."""
    tag = "" if not spinor else ("up" if spin == 0 else "down")
    return f"{seedname}{tag}_{w + 1:05d}.xsf"


def write_xsf_datagrid(path, data: np.ndarray, origin, axes, lattice: Optional[np.ndarray] = None) -> None:
    """data [NX, NY, NZ] (real) on the grid r = origin + sum_p (X_p / N_p) axes[p]; axes[p] is
    the p-th spanning vector of the whole grid (the supercell), lattice the unit cell (rows) for
    the CRYSTAL block (defaults to axes)."""
    data = np.asarray(data, dtype=float)
    nx, ny, nz = data.shape
    lat = np.asarray(axes if lattice is None else lattice, dtype=float).reshape(3, 3)
    axes = np.asarray(axes, dtype=float).reshape(3, 3)
    head = [" #", " # real-space Wannier function on a periodic grid", " #", "", "CRYSTAL", "PRIMVEC"]
    head += ["  " + " ".join(f"{x:.10f}" for x in lat[p]) for p in range(3)]
    head += ["CONVVEC"] + ["  " + " ".join(f"{x:.10f}" for x in lat[p]) for p in range(3)]
    head += ["PRIMCOORD", "  1  1", "X  0.0 0.0 0.0", "", "BEGIN_BLOCK_DATAGRID_3D", "  wannier",
             "BEGIN_DATAGRID_3D_wannier"]
    while len(head) < 22:
        head.insert(3, " #")
    assert len(head) == 22
    vals = data.transpose(2, 1, 0).reshape(-1)   # x fastest, then y, then z
    with open(path, "w") as fh:
        fh.write("\n".join(head) + "\n")
        fh.write(f"  {nx} {ny} {nz}\n")
        fh.write("  " + " ".join(f"{x:.10f}" for x in np.asarray(origin, dtype=float)) + "\n")
        for p in range(3):
            fh.write("  " + " ".join(f"{x:.10f}" for x in axes[p]) + "\n")
        for i in range(0, vals.size, 6):
            fh.write(" " + " ".join(f"{x:.8e}" for x in vals[i:i + 6]) + "\n")
        fh.write("END_DATAGRID_3D\nEND_BLOCK_DATAGRID_3D\n")


def read_xsf_datagrid(path):
    """(data [NX, NY, NZ], origin (3,), axes (3, 3): row p = spanning vector p) of the first
    DATAGRID_3D block of an XSF file."""
    with open(path) as fh:
        text = fh.read()
    pos = text.find("BEGIN_DATAGRID_3D")
    if pos < 0:
        raise ValueError(f"{path}: no BEGIN_DATAGRID_3D block")
    body = text[pos:].split("\n", 1)[1]
    end = body.find("END_DATAGRID_3D")
    tok = body[:end if end >= 0 else len(body)].split()
    nx, ny, nz = (int(float(t)) for t in tok[:3])
    origin = np.array([float(t) for t in tok[3:6]])
    axes = np.array([float(t) for t in tok[6:15]]).reshape(3, 3)
    vals = np.array([float(t) for t in tok[15:15 + nx * ny * nz]])
    if vals.size != nx * ny * nz:
        raise ValueError(f"{path}: {vals.size} grid values, {nx * ny * nz} expected")
    return vals.reshape(nz, ny, nx).transpose(2, 1, 0).copy(), origin, axes


def read_wannier_xsf(seedname: str, nw: int, spinor: bool = False):
    """All functions of a seedname: (data [n_spin_files, nw, NX, NY, NZ], origin, axes), the files
    in the reference's order (spin channel, then function)."""
    out, origin, axes = [], None, None
    for spin in range(2 if spinor else 1):
        row = []
        for w in range(nw):
            d, o, a = read_xsf_datagrid(xsf_name(seedname, w, spinor, spin))
            if origin is None:
                origin, axes = o, a
            row.append(d)
        out.append(row)
    return np.asarray(out), origin, axes
