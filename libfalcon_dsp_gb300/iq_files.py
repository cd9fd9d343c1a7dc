"""Sample files of the int16 front end: libfalcon_dsp's complex data files
(src/utilities/falcon_dsp_utils.cc:534-742, file_type_e in
hdr/utilities/falcon_dsp_utils.h:75-79).

* BINARY: interleaved little-endian (re, im) pairs, int16 ("<2h" per sample,
  the format SDR captures use) or float32.
* ASCII: one "re im" pair per line.

The reader decodes each int16 as little-endian two's complement.  (The
reference's BINARY int16 reader ORs a plain `char` low byte into the sample,
which on hosts where char is signed turns every sample whose low byte is
>= 0x80 into one with a high byte of 0xff; files written by its writer, and
by this module, hold the plain little-endian values.)

read_complex_data_from_file returns an (N, 2) int16 array for int16 data, the
layout the library's int16 entry points take directly (fdsp_*_apply_ci16).
"""
from __future__ import annotations

import numpy as np

BINARY, ASCII = 0, 1


def write_complex_data_to_file(file_name: str, file_type: int, data) -> bool:
    """complex int16 data as an (N, 2) int16 array, or complex64 data."""
    a = np.asarray(data)
    if a.dtype == np.int16:
        pairs = a.reshape(-1, 2).astype("<i2")
    else:
        c = a.astype(np.complex64).reshape(-1)
        pairs = np.stack([c.real, c.imag], axis=1).astype("<f4")
    try:
        if file_type == BINARY:
            pairs.tofile(file_name)
        elif file_type == ASCII:
            fmt = "%d %d" if a.dtype == np.int16 else "%.9g %.9g"
            np.savetxt(file_name, pairs, fmt=fmt)
        else:
            return False
    except OSError:
        return False
    return True


def read_complex_data_from_file(file_name: str, file_type: int, dtype=np.int16):
    """(N, 2) int16 array for dtype int16, complex64 array for float data;
    None where the reference returns false (missing file, bad type)."""
    try:
        if file_type == BINARY:
            raw = np.fromfile(file_name, dtype="<i2" if dtype == np.int16 else "<f4")
            raw = raw[: raw.size - raw.size % 2].reshape(-1, 2)
        elif file_type == ASCII:
            raw = np.loadtxt(file_name, dtype=np.float64, ndmin=2).reshape(-1, 2)
        else:
            return None
    except OSError:
        return None
    if dtype == np.int16:
        return raw.astype(np.int16)
    return (raw[:, 0] + 1j * raw[:, 1]).astype(np.complex64)


__all__ = ["BINARY", "ASCII", "write_complex_data_to_file", "read_complex_data_from_file"]
