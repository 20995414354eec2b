"""Single-file NIfTI-1 (.nii / .nii.gz) reading and writing, in process.

The reference reads single-file NIfTI-1 images through `system("gunzip")`
and a raw 352-byte header read (read_data.cpp:187-247) and writes FLOAT64
images with 2 mm voxels before gzipping them through `system("gzip")`
(nifti1_read_write.cpp:198-322).  This module does both with Python's
gzip, following the NIfTI-1 header layout (348-byte header, 4-byte
extension flag, data at vox_offset), either byte order.
"""
from __future__ import annotations

import gzip
import struct
from dataclasses import dataclass
from pathlib import Path

import numpy as np

# NIfTI-1 datatype codes
UINT8, INT16, INT32, FLOAT32, FLOAT64 = 2, 4, 8, 16, 64
INT8, UINT16, UINT32, INT64, UINT64 = 256, 512, 768, 1024, 1280
_DTYPES = {UINT8: "u1", INT16: "i2", INT32: "i4", FLOAT32: "f4", FLOAT64: "f8",
           INT8: "i1", UINT16: "u2", UINT32: "u4", INT64: "i8", UINT64: "u8"}
NAMES = {UINT8: "NIFTI_TYPE_UINT8", FLOAT32: "NIFTI_TYPE_FLOAT32",
         FLOAT64: "NIFTI_TYPE_FLOAT64", INT16: "NIFTI_TYPE_INT16"}


class NiftiError(ValueError):
    pass


@dataclass
class NiftiImage:
    data: np.ndarray          # [Z][Y][X] (x fastest in the file)
    datatype: int
    pixdim: tuple
    dims: tuple               # (X, Y, Z)


def _open(path: Path):
    raw = path.read_bytes()
    if raw[:2] == b"\x1f\x8b":
        raw = gzip.decompress(raw)
    return raw


def read_nifti(path) -> NiftiImage:
    path = Path(path)
    if not path.exists():
        raise NiftiError(f"{path}: no such file")
    raw = _open(path)
    if len(raw) < 348:
        raise NiftiError(f"{path}: shorter than a NIfTI-1 header")
    for endian in "<>":
        if struct.unpack(endian + "i", raw[:4])[0] == 348:
            break
    else:
        raise NiftiError(f"{path}: not a NIfTI-1 file (sizeof_hdr != 348)")
    dim = struct.unpack(endian + "8h", raw[40:56])
    datatype, bitpix = struct.unpack(endian + "2h", raw[70:74])
    pixdim = struct.unpack(endian + "8f", raw[76:108])
    vox_offset = int(struct.unpack(endian + "f", raw[108:112])[0])
    magic = raw[344:348]
    if magic[:3] != b"n+1":
        raise NiftiError(f"{path}: not a single-file NIfTI-1 image (magic {magic!r})")
    if dim[0] < 3 or any(d < 1 for d in dim[1:4]):
        raise NiftiError(f"{path}: bad dimensions {dim}")
    if datatype not in _DTYPES:
        raise NiftiError(f"{path}: unsupported datatype {datatype}")
    X, Y, Z = dim[1], dim[2], dim[3]
    n = X * Y * Z
    dt = np.dtype(_DTYPES[datatype]).newbyteorder(endian)
    off = max(vox_offset, 352)
    if len(raw) < off + n * dt.itemsize:
        raise NiftiError(f"{path}: truncated image data")
    data = np.frombuffer(raw, dtype=dt, count=n, offset=off).astype(dt.newbyteorder("="))
    return NiftiImage(data.reshape(Z, Y, X), datatype, pixdim[1:4], (X, Y, Z))


def nifti_bytes(data_xyz_fastest: np.ndarray, dims, datatype=FLOAT64,
                pixdim=(2.0, 2.0, 2.0)) -> bytes:
    """A single-file NIfTI-1 image as the reference writes it
    (nifti1_read_write.cpp:229-254): 3-D, FLOAT64 by default, 2 mm voxels,
    vox_offset 352, mm units, magic "n+1"."""
    X, Y, Z = dims
    hdr = bytearray(348)
    struct.pack_into("<i", hdr, 0, 348)
    struct.pack_into("<8h", hdr, 40, 3, X, Y, Z, 1, 0, 0, 0)
    dt = np.dtype(_DTYPES[datatype])
    struct.pack_into("<2h", hdr, 70, datatype, dt.itemsize * 8)
    struct.pack_into("<8f", hdr, 76, 0.0, *pixdim, 0.0, 0.0, 0.0, 0.0)
    struct.pack_into("<f", hdr, 108, 352.0)
    hdr[123] = 2  # NIFTI_UNITS_MM
    hdr[344:348] = b"n+1\x00"
    body = np.ascontiguousarray(data_xyz_fastest, dtype=dt.newbyteorder("<")).tobytes()
    if len(body) != X * Y * Z * dt.itemsize:
        raise NiftiError("data size does not match the dimensions")
    return bytes(hdr) + b"\x00\x00\x00\x00" + body


def write_nifti(path, data, dims, datatype=FLOAT64, pixdim=(2.0, 2.0, 2.0)):
    """Writes `path` (.nii or .nii.gz); data in file order (x fastest)."""
    path = Path(path)
    blob = nifti_bytes(np.asarray(data).reshape(-1), dims, datatype, pixdim)
    if path.suffix == ".gz":
        with gzip.open(path, "wb", compresslevel=6) as f:
            f.write(blob)
    else:
        path.write_bytes(blob)
