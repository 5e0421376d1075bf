"""Writes tests/golden/mrc2014_fei1_stack.mrc byte by byte from the published
MRC2014 specification (the 256 four-byte words of the main header, by word
number) and the FEI1 extended-header record layout (version 2, 768-byte
records), with nothing from guanaco_gb300.mrc: the fixture pins that module's
reading and writing to the format itself.

    python tests/golden/make_mrc_fixture.py

The file: a 3-tilt stack of 4 x 6 float32 images (mode 2, space group 0, an
image stack), pixel size 1.35 A, FEI1 records with the "Alpha tilt" and
"Defocus" fields the reference's file entry points read
(src/guanaco/detail/reconstruct.py:246-292, correct.py:375-471).
"""
import os
import struct

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PATH = os.path.join(HERE, "mrc2014_fei1_stack.mrc")

T, NY, NX = 3, 4, 6
PIXEL = 1.35
TILTS = (-30.0, 0.0, 30.0)
DEFOCUS = 25000.0
RECORD = 768


def data():
    return (np.arange(T * NY * NX, dtype=np.float32).reshape(T, NY, NX) * 0.5 - 7.0)


def main_header(d):
    w = [b"\0" * 4] * 256  # words 1..256 at w[0..255]
    i4 = lambda v: struct.pack("<i", v)  # noqa: E731
    f4 = lambda v: struct.pack("<f", v)  # noqa: E731
    w[0], w[1], w[2], w[3] = i4(NX), i4(NY), i4(T), i4(2)        # NX NY NZ MODE (2: float32)
    w[4], w[5], w[6] = i4(0), i4(0), i4(0)                       # NXSTART NYSTART NZSTART
    w[7], w[8], w[9] = i4(NX), i4(NY), i4(1)                     # MX MY MZ (image stack: MZ 1)
    w[10], w[11], w[12] = f4(PIXEL * NX), f4(PIXEL * NY), f4(PIXEL * 1)  # CELLA (A)
    w[13], w[14], w[15] = f4(90.0), f4(90.0), f4(90.0)           # CELLB (degrees)
    w[16], w[17], w[18] = i4(1), i4(2), i4(3)                    # MAPC MAPR MAPS
    w[19], w[20], w[21] = f4(float(d.min())), f4(float(d.max())), f4(float(d.mean()))
    w[22] = i4(0)                                                # ISPG: image stack
    w[23] = i4(T * RECORD)                                       # NSYMBT
    # words 25-49: EXTRA; bytes 104-107 EXTTYP, 108-111 NVERSION
    w[26] = b"FEI1"
    w[27] = i4(20140)
    w[49], w[50], w[51] = f4(0.0), f4(0.0), f4(0.0)              # ORIGIN
    w[52] = b"MAP "                                              # MAP
    w[53] = bytes((0x44, 0x44, 0x00, 0x00))                      # MACHST: little endian
    w[54] = f4(float(d.std()))                                   # RMS
    w[55] = i4(1)                                                # NLABL
    label = b"fixture: MRC2014 + FEI1, written from the specification".ljust(80, b" ")
    for k in range(20):                                          # LABEL 1 (words 57-76)
        w[56 + k] = label[4 * k:4 * k + 4]
    head = b"".join(w)
    assert len(head) == 1024
    return head


def fei1_record(tilt):
    r = bytearray(RECORD)
    struct.pack_into("<i", r, 0, RECORD)       # Metadata size
    struct.pack_into("<i", r, 4, 2)            # Metadata version
    struct.pack_into("<d", r, 100, tilt)       # Alpha tilt (degrees)
    struct.pack_into("<d", r, 220, DEFOCUS)    # Defocus (A)
    return bytes(r)


def write(path=PATH):
    d = data()
    with open(path, "wb") as f:
        f.write(main_header(d))
        for t in TILTS:
            f.write(fei1_record(t))
        f.write(d.astype("<f4").tobytes())
    return path


if __name__ == "__main__":
    print(write())
