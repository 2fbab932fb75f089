"""The film's way out: tonemapping (Tonemapper::map, src/tonemapper.cpp:31-56)
and the writers of --save-exr / --save-img / --save-mat (src/main.cpp:223-265)."""
import ctypes as C
import os

import numpy as np

from . import check, lib


def tonemap(film, gamma=2.2):
    """(H, W, 3) BGR float film -> (H, W, 3) RGB uint8 (host)."""
    film = np.ascontiguousarray(film, np.float32)
    out = np.zeros(film.shape, np.uint8)
    check(lib().gbrt_tonemap(film.ctypes.data_as(C.c_void_p), film.shape[1], film.shape[0], gamma,
                             out.ctypes.data_as(C.c_void_p)))
    return out


def write_image(path, film, gamma=2.2):
    """Writes by extension: .exr, .pfm, .hdr, .m, or .png / .ppm / .bmp (tonemapped)."""
    film = np.ascontiguousarray(film, np.float32)
    check(lib().gbrt_write_image(os.fsencode(path), film.ctypes.data_as(C.c_void_p), film.shape[1],
                                 film.shape[0], gamma))
    return path
