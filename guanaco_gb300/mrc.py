"""MRC2014 tilt series and volumes, memory mapped.

The reference reads and writes its files through the ``mrcfile`` package
(src/guanaco/detail/reconstruct.py:216-402, src/guanaco/detail/correct.py:
321-473), which is not a dependency here; this module implements the parts of
the MRC2014 format those functions use:

* the 1024-byte main header (little-endian): sizes, data mode, sampling
  (mx, my, mz), cell dimensions (voxel size = cell / sampling), space group
  (0 image stack, 1 volume, 401 stack of volumes), extended-header size and
  type, origin, ``MAP `` tag, machine stamp, statistics and labels;
* data modes 0 (int8), 1 (int16), 2 (float32), 4 (complex64: CTF images), 6
  (uint16) and 12 (float16),
  read as arrays of that type, X fastest;
* the FEI1 extended header: one record per image (per tilt and defocus for a
  corrected stack) whose first int32 is the record size; the reference uses
  the float64 fields "Alpha tilt" (degrees, byte 100 of the record) and
  "Defocus" (A, byte 220).

A stack of volumes (space group 401, mz slices per volume) maps to a 4D array
(nz / mz, mz, ny, nx): the corrected stack (tilts, defoci, height, width).
"""
from __future__ import annotations

import os

import numpy as np

MAIN_HEADER = np.dtype([
    ("nx", "<i4"), ("ny", "<i4"), ("nz", "<i4"), ("mode", "<i4"),
    ("nxstart", "<i4"), ("nystart", "<i4"), ("nzstart", "<i4"),
    ("mx", "<i4"), ("my", "<i4"), ("mz", "<i4"),
    ("cella", "<f4", 3), ("cellb", "<f4", 3),
    ("mapc", "<i4"), ("mapr", "<i4"), ("maps", "<i4"),
    ("dmin", "<f4"), ("dmax", "<f4"), ("dmean", "<f4"),
    ("ispg", "<i4"), ("nsymbt", "<i4"),
    ("extra1", "V8"), ("exttyp", "S4"), ("nversion", "<i4"), ("extra2", "V84"),
    ("origin", "<f4", 3), ("map", "S4"), ("machst", "u1", 4), ("rms", "<f4"),
    ("nlabl", "<i4"), ("label", "S80", 10),
])
assert MAIN_HEADER.itemsize == 1024

MODES = {0: np.dtype("i1"), 1: np.dtype("<i2"), 2: np.dtype("<f4"), 4: np.dtype("<c8"),
         6: np.dtype("<u2"), 12: np.dtype("<f2")}
MODE_OF = {v: k for k, v in MODES.items()}

# FEI1 extended-header record: the fields the reference uses, at their byte
# offsets, padded to the record size of version-2 records (768 bytes)
FEI1_RECORD_SIZE = 768
FEI1_RECORD = np.dtype({"names": ["Metadata size", "Metadata version", "Alpha tilt", "Defocus"],
                        "formats": ["<i4", "<i4", "<f8", "<f8"],
                        "offsets": [0, 4, 100, 220], "itemsize": FEI1_RECORD_SIZE})


class MrcFile:
    """An open MRC file: ``header`` (numpy record of MAIN_HEADER), ``data``
    (memory-mapped array), ``extended_header`` (FEI1 records shaped like the
    images, or None) and ``voxel_size`` (dict x, y, z in A)."""

    def __init__(self, path, header, data, extended_header, writable):
        self.path = path
        self.header = header
        self.data = data
        self.extended_header = extended_header
        self._writable = writable

    @property
    def voxel_size(self):
        h = self.header
        m = [max(int(h["mx"]), 1), max(int(h["my"]), 1), max(int(h["mz"]), 1)]
        c = h["cella"]
        return {"x": float(c[0]) / m[0], "y": float(c[1]) / m[1], "z": float(c[2]) / m[2]}

    def set_voxel_size(self, size):
        sx, sy, sz = (size, size, size) if np.isscalar(size) else size
        h = self.header
        h["cella"] = (sx * h["mx"], sy * h["my"], sz * h["mz"])

    def close(self):
        if self._writable:
            d = None
            if self.data.size < (1 << 26):  # statistics of the magnitude for complex data
                d = np.abs(self.data) if np.iscomplexobj(self.data) else self.data
                d = np.asarray(d, dtype=np.float64)
            h = self.header
            if d is not None and d.size:
                h["dmin"], h["dmax"], h["dmean"] = d.min(), d.max(), d.mean()
                h["rms"] = d.std()
            with open(self.path, "r+b") as f:
                f.write(h.tobytes())
                if self.extended_header is not None:
                    f.write(self.extended_header.tobytes())
            self.data.flush()
            self._writable = False

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def _shape(h):
    nx, ny, nz = int(h["nx"]), int(h["ny"]), int(h["nz"])
    if int(h["ispg"]) == 401 and int(h["mz"]) > 0 and nz % int(h["mz"]) == 0:
        return (nz // int(h["mz"]), int(h["mz"]), ny, nx)
    return (ny, nx) if nz == 1 else (nz, ny, nx)


def open_mrc(path, mode="r"):
    """Open an existing file ("r" read only, "r+" read and write), memory mapped."""
    header = np.fromfile(path, dtype=MAIN_HEADER, count=1)[0].copy()
    if header["map"] != b"MAP ":
        raise ValueError(f"{path}: not an MRC2014 file (no 'MAP ' tag)")
    if int(header["mode"]) not in MODES:
        raise ValueError(f"{path}: unsupported MRC mode {int(header['mode'])}")
    shape = _shape(header)
    nsym = int(header["nsymbt"])
    ext = None
    if nsym > 0 and header["exttyp"] == b"FEI1":
        raw = np.fromfile(path, dtype=np.uint8, count=nsym, offset=1024)
        size = int(np.frombuffer(raw[:4].tobytes(), "<i4")[0]) or FEI1_RECORD_SIZE
        n = nsym // size
        rec = np.dtype({"names": FEI1_RECORD.names,
                        "formats": [FEI1_RECORD.fields[k][0] for k in FEI1_RECORD.names],
                        "offsets": [FEI1_RECORD.fields[k][1] for k in FEI1_RECORD.names],
                        "itemsize": size})
        ext = np.frombuffer(raw[: n * size].tobytes(), dtype=rec).copy()
        images = shape[:-2]
        if int(np.prod(images)) == n:
            ext = ext.reshape(images)
    data = np.memmap(path, dtype=MODES[int(header["mode"])], mode=mode, offset=1024 + nsym,
                     shape=shape)
    return MrcFile(path, header, data, ext, writable=(mode != "r"))


def new_mrc(path, shape, dtype=np.float32, voxel_size=1.0, fei1=False, overwrite=True):
    """Create a file of the given data shape: 2D image, 3D image stack
    (``fei1``: one FEI1 record per image) or volume (space group 1 when
    ``fei1`` is False), or 4D stack of volumes (tilts, defoci, height, width),
    memory mapped for writing."""
    if os.path.exists(path) and not overwrite:
        raise FileExistsError(path)
    dtype = np.dtype(dtype).newbyteorder("<") if np.dtype(dtype).byteorder == ">" else np.dtype(dtype)
    if dtype not in MODE_OF:
        raise ValueError(f"no MRC mode for {dtype}")
    shape = tuple(int(s) for s in shape)
    h = np.zeros((), dtype=MAIN_HEADER)
    if len(shape) == 4:
        nv, mz, ny, nx = shape
        nz, ispg = nv * mz, 401
    elif len(shape) == 3:
        nz, ny, nx = shape
        mz, ispg = (1, 0) if fei1 else (nz, 1)
    elif len(shape) == 2:
        (ny, nx), nz, mz, ispg = shape, 1, 1, 0
    else:
        raise ValueError("MRC data is 2D, 3D or 4D")
    h["nx"], h["ny"], h["nz"], h["mode"] = nx, ny, nz, MODE_OF[dtype]
    h["mx"], h["my"], h["mz"] = nx, ny, mz
    h["cellb"] = (90.0, 90.0, 90.0)
    h["mapc"], h["mapr"], h["maps"] = 1, 2, 3
    h["ispg"] = ispg
    h["map"] = b"MAP "
    h["machst"] = (0x44, 0x44, 0x00, 0x00)
    h["nversion"] = 20140
    ext = None
    if fei1:
        n_images = int(np.prod(shape[:-2]))
        ext = np.zeros(shape[:-2], dtype=FEI1_RECORD)
        ext["Metadata size"] = FEI1_RECORD_SIZE
        h["exttyp"] = b"FEI1"
        h["nsymbt"] = n_images * FEI1_RECORD_SIZE
    mf = MrcFile(path, h, None, ext, writable=True)
    mf.set_voxel_size(voxel_size)
    with open(path, "wb") as f:
        f.write(h.tobytes())
        if ext is not None:
            f.write(ext.tobytes())
        f.truncate(1024 + int(h["nsymbt"]) + int(np.prod(shape)) * dtype.itemsize)
    mf.data = np.memmap(path, dtype=dtype, mode="r+", offset=1024 + int(h["nsymbt"]), shape=shape)
    return mf


def fei1_angles_deg(mf):
    """Per-tilt "Alpha tilt" (degrees) of an FEI1 image or corrected stack."""
    ext = mf.extended_header
    if ext is None:
        raise ValueError(f"{mf.path}: no FEI1 extended header")
    return np.asarray(ext["Alpha tilt"] if ext.ndim == 1 else ext[:, 0]["Alpha tilt"], np.float64)


def fei1_defocus(mf):
    """Per-slab "Defocus" (A) of an FEI1 corrected stack (tilts, defoci, ...)."""
    ext = mf.extended_header
    if ext is None or ext.ndim != 2:
        raise ValueError(f"{mf.path}: no per-slab FEI1 records")
    return np.asarray(ext[0, :]["Defocus"], np.float64)
