"""TEST INFRASTRUCTURE ONLY: ctypes access to the CPU oracles.

* ``Port`` wraps ``_build/liblbm_oracle.so``, the C restatement of the serial
  reference's time step (lbm_oracle.c).  It is built on every host.
* ``Ref`` wraps ``_ref/libserialref.so``, the unmodified serial reference
  (mate-szoke/ParallelLbmCranfield serial/) linked with ref_harness.c.  It
  exists only where the reference sources were present at build time.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs import
this module.  Arrays are numpy, cell-major (``F[cell, k]``), cells row-major
``j * n + i`` as in the reference.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "liblbm_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libserialref.so")
# The reference checkout (mate-szoke/ParallelLbmCranfield) is named by the
# LBM_REFERENCE_DIR environment variable; where it is unset or absent, the
# reference harness is not built and the tests that need it skip.
REF_ROOT = os.environ.get("LBM_REFERENCE_DIR", "/root/reference")
REF_SRC = os.path.join(REF_ROOT, "serial")
REF_CASES = os.path.join(REF_ROOT, "cases")

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_fp = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")


def build(ref=None):
    """Build the port (always) and the reference harness (when its sources exist)."""
    subprocess.check_call(["make", "-s", "-C", HERE, "port"])
    if ref is None:
        ref = os.path.isdir(REF_SRC)
    if ref:
        subprocess.check_call(["make", "-s", "-C", HERE, "ref", f"REF_DIR={REF_SRC}"])


def ref_available():
    return os.path.exists(REF_SO)


class or_params(C.Structure):
    _fields_ = [("uavg", C.c_float), ("vavg", C.c_float), ("rho_ini", C.c_float),
                ("viscosity", C.c_float), ("inlet_profile", C.c_int), ("model", C.c_int),
                ("curved", C.c_int), ("outlet", C.c_int), ("drag_id", C.c_int),
                ("rho_out", C.c_double)]


_port_lib = None
_ref_lib = None


def _load_port():
    global _port_lib
    if _port_lib is None:
        if not os.path.exists(PORT_SO):
            build(ref=False)
        L = C.CDLL(PORT_SO)
        L.or_create.restype = C.c_void_p
        L.or_create.argtypes = [_fp, C.c_int, _fp, C.c_int, C.POINTER(or_params)]
        L.or_read_mesh.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(C.POINTER(C.c_float)),
                                   C.POINTER(C.c_int), C.POINTER(C.POINTER(C.c_float)),
                                   C.POINTER(C.c_int)]
        L.or_free.argtypes = [C.c_void_p]
        L.or_destroy.argtypes = [C.c_void_p]
        L.or_dims.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.or_constants.argtypes = [C.c_void_p, _dp]
        L.or_get_init.argtypes = [C.c_void_p, _ip, _dp]
        L.or_set_state.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.or_run.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        L.or_run.restype = C.c_int
        L.or_get.argtypes = [C.c_void_p] + [C.c_void_p] * 7
        L.or_diagnostics.argtypes = [C.c_void_p, _dp]
        _port_lib = L
    return _port_lib


def _load_ref():
    global _ref_lib
    if _ref_lib is None:
        L = C.CDLL(REF_SO)
        L.ref_create.restype = C.c_void_p
        L.ref_create.argtypes = [C.c_char_p, C.c_char_p, C.c_float, C.c_float, C.c_float,
                                 C.c_float, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
        L.ref_dims.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.ref_constants.argtypes = [C.c_void_p, _dp]
        L.ref_get_init.argtypes = [C.c_void_p, _ip, _dp]
        L.ref_set_state.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.ref_run.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        L.ref_get.argtypes = [C.c_void_p] + [C.c_void_p] * 7
        L.ref_destroy.argtypes = [C.c_void_p]
        _ref_lib = L
    return _ref_lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def read_mesh(nodefile, connfile):
    """Parse mesh files exactly as the reference does (fscanf %f)."""
    L = _load_port()
    pn, pc = C.POINTER(C.c_float)(), C.POINTER(C.c_float)()
    nn, nc = C.c_int(), C.c_int()
    if L.or_read_mesh(nodefile.encode(), connfile.encode(), C.byref(pn), C.byref(nn),
                      C.byref(pc), C.byref(nc)) != 0:
        raise FileNotFoundError(nodefile)
    nodes = np.ctypeslib.as_array(pn, shape=(max(nn.value, 1), 5)).copy()[: nn.value]
    conns = np.ctypeslib.as_array(pc, shape=(max(nc.value, 1), 7)).copy()[: nc.value]
    L.or_free(C.cast(pn, C.c_void_p))
    L.or_free(C.cast(pc, C.c_void_p))
    return nodes, conns


class _Sim:
    def _alloc_get(self, fields):
        N = self.n * self.m
        out = {}
        for f in fields:
            out[f] = np.zeros((N, 9) if f in ("F", "METAF") else N, np.float64)
        return out

    def state(self):
        o = self._alloc_get(["F", "METAF", "rho", "u", "v", "drag", "lift"])
        self._get(*[_ptr(o[k]) for k in ("F", "METAF", "rho", "u", "v", "drag", "lift")])
        return o

    def set_state(self, F=None, rho=None, u=None, v=None):
        arrs = [None if a is None else np.ascontiguousarray(a, np.float64)
                for a in (F, rho, u, v)]
        self._set(*[_ptr(a) for a in arrs])

    def init_fields(self):
        N = self.n * self.m
        ints = np.zeros((N, 23), np.int32)
        reals = np.zeros((N, 14), np.float64)
        self._get_init(ints, reals)
        return ints, reals

    def constants(self):
        c = np.zeros(5)
        self._consts(c)
        return c


class Port(_Sim):
    """C restatement of the serial step; params mirror SetUpData.ini."""

    def __init__(self, nodes, conns, uavg, vavg, rho_ini, viscosity, inlet_profile=2,
                 model=1, curved=2, outlet=2, drag_id=0, rho_out=1.0):
        L = self.L = _load_port()
        p = or_params(uavg, vavg, rho_ini, viscosity, inlet_profile, model, curved, outlet,
                      drag_id, rho_out)
        nodes = np.ascontiguousarray(nodes, np.float32)
        conns = np.ascontiguousarray(conns, np.float32).reshape(-1, 7)
        self.h = L.or_create(nodes.reshape(-1), len(nodes), conns.reshape(-1), len(conns),
                             C.byref(p))
        if not self.h:
            raise ValueError("oracle: empty mesh")
        n, m = C.c_int(), C.c_int()
        L.or_dims(self.h, C.byref(n), C.byref(m))
        self.n, self.m = n.value, m.value

    def _get(self, *a):
        self.L.or_get(self.h, *a)

    def _set(self, *a):
        self.L.or_set_state(self.h, *a)

    def _get_init(self, i, r):
        self.L.or_get_init(self.h, i, r)

    def _consts(self, c):
        self.L.or_constants(self.h, c)

    def run(self, nsteps, want_resid=True):
        r = np.zeros((max(nsteps, 1), 4)) if want_resid else None
        st = self.L.or_run(self.h, nsteps, _ptr(r))
        return st, (r[:nsteps] if want_resid else None)

    def diagnostics(self):
        d = np.zeros(6)
        self.L.or_diagnostics(self.h, d)
        return d

    def close(self):
        if self.h:
            self.L.or_destroy(self.h)
            self.h = None

    __del__ = close


class Ref(_Sim):
    """The unmodified serial reference, driven step by step."""

    def __init__(self, nodefile, connfile, uavg, vavg, rho_ini, viscosity, inlet_profile=2,
                 model=1, curved=2, outlet=2, drag_id=0):
        L = self.L = _load_ref()
        self.h = L.ref_create(nodefile.encode(), connfile.encode(), uavg, vavg, rho_ini,
                              viscosity, inlet_profile, model, curved, outlet, drag_id)
        if not self.h:
            raise FileNotFoundError(nodefile)
        n, m = C.c_int(), C.c_int()
        L.ref_dims(self.h, C.byref(n), C.byref(m))
        self.n, self.m = n.value, m.value

    def _get(self, *a):
        self.L.ref_get(self.h, *a)

    def _set(self, *a):
        self.L.ref_set_state(self.h, *a)

    def _get_init(self, i, r):
        self.L.ref_get_init(self.h, i, r)

    def _consts(self, c):
        self.L.ref_constants(self.h, c)

    def run(self, nsteps, want_resid=True):
        r = np.zeros((max(nsteps, 1), 4)) if want_resid else None
        self.L.ref_run(self.h, nsteps, _ptr(r))
        return 0, (r[:nsteps] if want_resid else None)

    def close(self):
        if self.h:
            self.L.ref_destroy(self.h)
            self.h = None

    __del__ = close


def feq_rest(rho0, N):
    """f = f_eq(rho0, 0, 0), cell-major."""
    w = np.array([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4)
    return np.tile(rho0 * w, (N, 1))
