"""stem3 .img files: the reference's image format (libs/imagelib_fftw3.h:30-66).

Layout (little endian): a 56-byte header of eight int32 -- headerSize (56),
paramSize, commentSize, nx, ny, complexFlag, dataSize, version -- and three
float64 -- t (thickness), dx, dy; then paramSize float64 parameters, the
comment (commentSize bytes, no terminator), then nx*ny float32 (real) or
complex64 values in [nx][ny] order (libs/imagelib_fftw3.cpp:71-110).

The writer produces files the reference's ReadImage accepts; the reader
uses the true parameter offset (8 bytes per parameter).  The reference's own
ReadImage seeks 2 bytes per parameter (libs/imagelib_fftw3.cpp:175), so it
only reads parameter-less files correctly -- which are the files it reads
back itself (diffAvg_*.img, mulswav_*.img).
"""
import struct

import numpy as np

HEADER = struct.Struct("<8i3d")
VERSION = 1  # the image-format version of libs/imagelib_fftw3.cpp:26


class Image:
    def __init__(self, data, t=0.0, dx=1.0, dy=1.0, params=(), comment="", version=0):
        self.data = data
        self.t, self.dx, self.dy = float(t), float(dx), float(dy)
        self.params = np.asarray(params, dtype=np.float64)
        self.comment = comment
        self.version = version

    @property
    def complex(self):
        return np.iscomplexobj(self.data)


def read_img(path):
    with open(path, "rb") as f:
        raw = f.read()
    (hs, nparam, ncomment, nx, ny, cflag, dsize, version, t, dx, dy) = HEADER.unpack_from(raw, 0)
    if hs != 56:
        raise ValueError("%s: not a stem3 .img file (header size %d)" % (path, hs))
    off = 56
    params = np.frombuffer(raw, dtype="<f8", count=nparam, offset=off).copy()
    off += 8 * nparam
    comment = raw[off:off + ncomment].decode("latin-1")
    off += ncomment
    if cflag:
        if dsize == 8:
            data = np.frombuffer(raw, dtype="<c8", count=nx * ny, offset=off)
        elif dsize == 16:
            data = np.frombuffer(raw, dtype="<c16", count=nx * ny, offset=off)
        else:
            raise ValueError("%s: complex data size %d" % (path, dsize))
    else:
        dt = {4: "<f4", 8: "<f8"}.get(dsize)
        if dt is None:
            raise ValueError("%s: real data size %d" % (path, dsize))
        data = np.frombuffer(raw, dtype=dt, count=nx * ny, offset=off)
    return Image(data.reshape(nx, ny).copy(), t, dx, dy, params, comment, version)


def write_img(path, data, t=0.0, dx=1.0, dy=1.0, params=(), comment=""):
    """Write a real (float32) or complex (complex64) [nx][ny] array.  A
    trailing axis of length 2 is read as (re, im)."""
    a = np.asarray(data)
    if a.ndim == 3 and a.shape[-1] == 2 and not np.iscomplexobj(a):
        a = a[..., 0].astype(np.float32) + 1j * a[..., 1].astype(np.float32)
    if np.iscomplexobj(a):
        a = np.ascontiguousarray(a, dtype=np.complex64)
        cflag, dsize = 1, 8
    else:
        a = np.ascontiguousarray(a, dtype=np.float32)
        cflag, dsize = 0, 4
    nx, ny = a.shape
    params = np.asarray(params, dtype="<f8")
    cbytes = comment.encode("latin-1")
    hdr = HEADER.pack(56, len(params), len(cbytes), nx, ny, cflag, dsize, VERSION, float(t), float(dx),
                      float(dy))
    with open(path, "wb") as f:
        f.write(hdr)
        f.write(params.tobytes())
        f.write(cbytes)
        f.write(a.tobytes())
