"""ctypes wrapper of the FP64 elastic FD oracle (oracle/fwi_oracle.c) —
TEST INFRASTRUCTURE ONLY.  Arrays are numpy float64 in [z][x] layout."""
import ctypes

import numpy as np

from oracle import build_oracle

_lib = None


class _Shot(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int),
        ("nz", ctypes.c_int),
        ("nt", ctypes.c_int),
        ("h", ctypes.c_double),
        ("dt", ctypes.c_double),
        ("taper", ctypes.c_void_p),
        ("stf", ctypes.c_void_p),
        ("src_x", ctypes.c_int),
        ("src_z", ctypes.c_int),
        ("nrec", ctypes.c_int),
        ("rec_x", ctypes.c_void_p),
        ("rec_z", ctypes.c_void_p),
        ("nsrc", ctypes.c_int),
        ("msrc_x", ctypes.c_void_p),
        ("msrc_z", ctypes.c_void_p),
        ("moment", ctypes.c_void_p),
        ("mstf", ctypes.c_void_p),
        ("snapshot_interval", ctypes.c_int),
    ]


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build_oracle.build())
        _lib.fwi_forward.restype = ctypes.c_int
        _lib.fwi_forward.argtypes = [ctypes.c_void_p] * 8
        _lib.fwi_gradient.restype = ctypes.c_double
        _lib.fwi_gradient.argtypes = [ctypes.c_void_p] * 6 + [ctypes.c_double] + [ctypes.c_void_p] * 3
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class Shot:
    """One shot.  `src` is an explosive source's simulation cell (x, z) fed
    by `stf`, or, with `sources` = [(x, z, Mxx, Mzz, Mxz), ...] and `stf` of
    shape [len(sources)][nt], moment-tensor point sources (src unused).
    `snapshot_interval` k > 1 correlates the gradient at every k-th step."""

    def __init__(self, nx, nz, nt, h, dt, taper, stf, src, rec_x, rec_z, sources=None, snapshot_interval=1):
        self.taper = np.ascontiguousarray(taper, np.float64)
        self.stf = np.ascontiguousarray(stf, np.float64)
        self.rec_x = np.ascontiguousarray(rec_x, np.int32)
        self.rec_z = np.ascontiguousarray(rec_z, np.int32)
        if sources is None:
            self.s = _Shot(nx, nz, nt, h, dt, _p(self.taper).value, _p(self.stf).value, int(src[0]), int(src[1]),
                           len(self.rec_x), _p(self.rec_x).value, _p(self.rec_z).value, 0, None, None, None, None,
                           int(snapshot_interval))
        else:
            srcs = np.asarray(sources, np.float64).reshape(-1, 5)
            assert self.stf.shape == (len(srcs), nt)
            self.msrc_x = np.ascontiguousarray(srcs[:, 0], np.int32)
            self.msrc_z = np.ascontiguousarray(srcs[:, 1], np.int32)
            self.moment = np.ascontiguousarray(srcs[:, 2:5], np.float64)
            self.s = _Shot(nx, nz, nt, h, dt, _p(self.taper).value, None, 0, 0, len(self.rec_x),
                           _p(self.rec_x).value, _p(self.rec_z).value, len(srcs), _p(self.msrc_x).value,
                           _p(self.msrc_z).value, _p(self.moment).value, _p(self.stf).value, int(snapshot_interval))
        self.nt, self.nrec = nt, len(self.rec_x)

    def forward(self, rho, vp, vs):
        rvx = np.zeros((self.nt, self.nrec))
        rvz = np.zeros((self.nt, self.nrec))
        args = [np.ascontiguousarray(a, np.float64) for a in (rho, vp, vs)]
        rc = lib().fwi_forward(ctypes.byref(self.s), *[_p(a) for a in args], _p(rvx), _p(rvz), None, None)
        assert rc == 0
        return rvx, rvz

    def gradient(self, rho, vp, vs, obs_vx, obs_vz, w):
        args = [np.ascontiguousarray(a, np.float64) for a in (rho, vp, vs)]
        g = [np.zeros_like(args[0]) for _ in range(3)]
        chi = lib().fwi_gradient(ctypes.byref(self.s), *[_p(a) for a in args],
                                 _p(np.ascontiguousarray(obs_vx, np.float64)),
                                 _p(np.ascontiguousarray(obs_vz, np.float64)), float(w), *[_p(x) for x in g])
        return chi, g  # g = [g_rho, g_vp, g_vs]


def timed_shot(task):
    """CPU cost of one shot of the FP64 restatement: returns (forward seconds,
    forward + adjoint gradient seconds).  `task` = (nx, nz, nt, h, dt, taper,
    stf, src, rec_x, rec_z, rho, vp, vs); used as a process-pool task to time
    the CPU baseline on every host core at once."""
    import time

    nx, nz, nt, h, dt, taper, stf, src, rec_x, rec_z, rho, vp, vs = task
    shot = Shot(nx, nz, nt, h, dt, taper, stf, src, rec_x, rec_z)
    t0 = time.perf_counter()
    ovx, ovz = shot.forward(rho, vp, vs)
    t1 = time.perf_counter()
    shot.gradient(rho, vp * 1.01, vs, ovx, ovz, 1.0)
    t2 = time.perf_counter()
    return t1 - t0, t2 - t1
