"""GB300-native D2Q9 lattice-Boltzmann time step (ctypes front end).

The product is the C ABI in include/lbm_gb300.h, implemented by
liblbm_gb300.so (built in-tree by build.py).  This module loads that library
and wraps it for Python callers (tests, bench.py, the drop-in driver).  There
is no CPU fallback: without the library every call raises.

Arrays are numpy, cells row-major ``j * n + i`` like the reference's cell
array; ``f``/``metaf`` are cell-major ``[cell, k]``.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblbm_gb300.so")

LBM_OK, LBM_DIVERGED, LBM_IO, LBM_CUDA, LBM_TIMEOUT, LBM_INVALID, LBM_NOMEM = range(7)
FP64, FP32, FP16DEV, BF16DEV, FP16NEQ = range(5)
AB, AA = range(2)
BGKW, TRT, MRT = 1, 2, 3
PRECISIONS = {"fp64": FP64, "fp32": FP32, "fp16dev": FP16DEV, "bf16dev": BF16DEV,
              "fp16neq": FP16NEQ}
PATTERNS = {"ab": AB, "aa": AA}


class LbmError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{msg} (status {status})")
        self.status = status


class DivergedError(LbmError):
    pass


class lbm_mesh(C.Structure):
    _fields_ = [("nodes", C.POINTER(C.c_float)), ("num_nodes", C.c_int32),
                ("conns", C.POINTER(C.c_float)), ("num_conns", C.c_int32)]


class lbm_params(C.Structure):
    _fields_ = [("uavg", C.c_float), ("vavg", C.c_float), ("rho_ini", C.c_float),
                ("viscosity", C.c_float), ("inlet_profile", C.c_int32),
                ("collision_model", C.c_int32), ("curved_boundaries", C.c_int32),
                ("outlet_profile", C.c_int32), ("drag_lift_id", C.c_int32),
                ("precision", C.c_int32), ("pattern", C.c_int32), ("device", C.c_int32),
                ("rho_out", C.c_double), ("stream", C.c_void_p), ("tile_variant", C.c_int32)]


class lbm_diagnostics(C.Structure):
    _fields_ = [("iteration", C.c_int64), ("l2_full", C.c_double), ("du_rel", C.c_double),
                ("mass", C.c_double), ("momentum", C.c_double * 2),
                ("force", C.c_double * 2), ("max_speed", C.c_double)]


# every symbol include/lbm_gb300.h declares
EXPORTS = ["lbm_status_string", "lbm_last_error", "lbm_create", "lbm_destroy", "lbm_get_dims",
           "lbm_set_state", "lbm_step", "lbm_get_fields", "lbm_check", "lbm_check_noalloc",
           "lbm_get_info", "lbm_autotune",
           "lbm_inspect_mesh", "lbm_batch_create", "lbm_batch_destroy", "lbm_batch_set_rest", "lbm_batch_set_tile",
           "lbm_batch_set_launch",
           "lbm_batch_set_state",
           "lbm_batch_autotune", "lbm_batch_run", "lbm_batch_get_fields", "lbm_batch_dims",
           "lbm_batch_info", "lbm_mesh_read", "lbm_mesh_cavity", "lbm_mesh_channel", "lbm_mesh_write",
           "lbm_mesh_free", "lbm_sg_create", "lbm_sg_destroy", "lbm_sg_num_params",
           "lbm_sg_get_params", "lbm_sg_set_params", "lbm_sg_forward", "lbm_sg_loss_grads",
           "lbm_sg_adam_step", "lbm_sg_set_dataset", "lbm_sg_train", "lbm_sg_set_lr"]

_lib = None


def load():
    """Load liblbm_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: run parallellbmcranfield_gb300/build.py "
                           "(the CUDA library is required; there is no CPU fallback)")
    L = C.CDLL(LIB_PATH)
    vp, i32, dp = C.c_void_p, C.c_int32, C.c_void_p
    L.lbm_status_string.restype = C.c_char_p
    L.lbm_status_string.argtypes = [C.c_int]
    L.lbm_last_error.restype = C.c_char_p
    L.lbm_create.argtypes = [C.POINTER(lbm_mesh), C.POINTER(lbm_params), C.POINTER(vp)]
    L.lbm_destroy.argtypes = [vp]
    L.lbm_destroy.restype = None
    L.lbm_get_dims.argtypes = [vp, C.POINTER(i32), C.POINTER(i32)]
    L.lbm_set_state.argtypes = [vp, dp, dp, dp, dp]
    L.lbm_step.argtypes = [vp, i32, i32, dp]
    L.lbm_get_fields.argtypes = [vp, dp, dp, dp, dp, dp]
    L.lbm_check.argtypes = [vp, C.POINTER(lbm_diagnostics)]
    L.lbm_check_noalloc.argtypes = [vp, C.POINTER(lbm_diagnostics)]
    L.lbm_autotune.argtypes = [vp, i32, C.c_char_p, C.c_char_p, C.c_size_t]
    L.lbm_get_info.argtypes = [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(i32)]
    L.lbm_inspect_mesh.argtypes = [C.POINTER(lbm_mesh), C.POINTER(lbm_params), C.POINTER(i32),
                                   C.POINTER(i32), dp, dp, dp]
    L.lbm_batch_create.argtypes = [C.POINTER(lbm_mesh), C.POINTER(lbm_params), i32, C.POINTER(vp)]
    L.lbm_batch_destroy.argtypes = [vp]
    L.lbm_batch_destroy.restype = None
    L.lbm_batch_set_rest.argtypes = [vp]
    L.lbm_batch_set_tile.argtypes = [vp, i32]
    L.lbm_batch_set_launch.argtypes = [vp, i32, i32]
    L.lbm_batch_set_state.argtypes = [vp, i32, dp, dp, dp]
    L.lbm_batch_autotune.argtypes = [vp, i32, C.c_char_p, C.c_size_t]
    L.lbm_batch_run.argtypes = [vp, C.c_int64, i32, C.c_double, dp, dp, dp, C.POINTER(C.c_double)]
    L.lbm_batch_get_fields.argtypes = [vp, i32, dp, dp, dp]
    L.lbm_batch_dims.argtypes = [vp, i32, C.POINTER(i32), C.POINTER(i32)]
    L.lbm_batch_info.argtypes = [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(i32),
                                 C.POINTER(C.c_int64)]
    L.lbm_mesh_read.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(lbm_mesh)]
    L.lbm_mesh_cavity.argtypes = [i32, C.POINTER(lbm_mesh)]
    L.lbm_mesh_channel.argtypes = [i32, i32, i32, dp, dp, dp, C.POINTER(lbm_mesh)]
    L.lbm_mesh_write.argtypes = [C.POINTER(lbm_mesh), C.c_char_p, C.c_char_p]
    L.lbm_mesh_free.argtypes = [C.POINTER(lbm_mesh)]
    L.lbm_mesh_free.restype = None
    for name in EXPORTS:
        if name not in ("lbm_destroy", "lbm_mesh_free", "lbm_status_string", "lbm_last_error",
                        "lbm_batch_destroy"):
            getattr(L, name).restype = C.c_int
    _lib = L
    return L


def _check(status, what):
    if status != LBM_OK:
        L = load()
        msg = f"{what}: {L.lbm_status_string(status).decode()}: {L.lbm_last_error().decode()}"
        raise (DivergedError if status == LBM_DIVERGED else LbmError)(status, msg)


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Mesh:
    """A mesh in the reference's format, held as numpy arrays (nodes Nx5, conns Cx7)."""

    def __init__(self, nodes, conns):
        self.nodes = np.ascontiguousarray(nodes, np.float32).reshape(-1, 5)
        self.conns = np.ascontiguousarray(conns, np.float32).reshape(-1, 7)

    @staticmethod
    def _from_c(fn, *args):
        L = load()
        m = lbm_mesh()
        _check(fn(*args, C.byref(m)), fn.__name__)
        try:
            nodes = np.ctypeslib.as_array(m.nodes, shape=(max(m.num_nodes, 1), 5))[: m.num_nodes].copy()
            conns = (np.ctypeslib.as_array(m.conns, shape=(max(m.num_conns, 1), 7))[: m.num_conns].copy()
                     if m.num_conns > 0 else np.zeros((0, 7), np.float32))
        finally:
            L.lbm_mesh_free(C.byref(m))
        return Mesh(nodes, conns)

    @staticmethod
    def read(node_file, conn_file):
        L = load()
        return Mesh._from_c(L.lbm_mesh_read, str(node_file).encode(), str(conn_file).encode())

    @staticmethod
    def cavity(side):
        return Mesh._from_c(load().lbm_mesh_cavity, int(side))

    @staticmethod
    def channel(nx, ny, cylinders=()):
        cyl = np.asarray(cylinders, np.float64).reshape(-1, 3)
        cx, cy, r = (np.ascontiguousarray(cyl[:, i]) for i in range(3))
        return Mesh._from_c(load().lbm_mesh_channel, int(nx), int(ny), len(cyl), _ptr(cx),
                            _ptr(cy), _ptr(r))

    def write(self, node_file, conn_file):
        _check(load().lbm_mesh_write(C.byref(self.c_struct()), str(node_file).encode(),
                                     str(conn_file).encode()), "lbm_mesh_write")

    def c_struct(self):
        m = lbm_mesh()
        m.nodes = self.nodes.ctypes.data_as(C.POINTER(C.c_float))
        m.num_nodes = len(self.nodes)
        m.conns = self.conns.ctypes.data_as(C.POINTER(C.c_float))
        m.num_conns = len(self.conns)
        return m

    @property
    def shape(self):
        """(n, m) as CompDataNode derives it from the last node record."""
        return int(self.nodes[-1, 0]) + 1, int(self.nodes[-1, 1]) + 1


def make_params(uavg=0.05, vavg=0.0, rho_ini=1.0, viscosity=0.01, inlet_profile=2,
                collision_model=BGKW, curved_boundaries=2, outlet_profile=2, drag_lift_id=0,
                precision=FP64, pattern=AB, rho_out=1.0, device=0, stream=None, tile_variant=0):
    if isinstance(precision, str):
        precision = PRECISIONS[precision]
    if isinstance(pattern, str):
        pattern = PATTERNS[pattern]
    return lbm_params(uavg, vavg, rho_ini, viscosity, inlet_profile, collision_model,
                      curved_boundaries, outlet_profile, drag_lift_id, precision, pattern,
                      device, rho_out, stream, tile_variant)


def inspect_mesh(mesh, **params):
    """CellIni's per-cell decisions as lbm_create derives them (host only)."""
    L = load()
    p = make_params(**params)
    n, m = mesh.shape
    cls = np.zeros(n * m, np.uint8)
    flags = np.zeros(n * m, np.uint32)
    q = np.zeros((n * m, 9))
    nn, mm = C.c_int32(), C.c_int32()
    _check(L.lbm_inspect_mesh(C.byref(mesh.c_struct()), C.byref(p), C.byref(nn), C.byref(mm),
                              _ptr(cls), _ptr(flags), _ptr(q)), "lbm_inspect_mesh")
    return {"n": nn.value, "m": mm.value, "cls": cls, "flags": flags, "q": q}


class Solver:
    """One resident domain on one GPU (wraps lbm_ctx).

    Keyword arguments are the SetUpData.ini switches (uavg, vavg, rho_ini,
    viscosity, inlet_profile, collision_model, curved_boundaries,
    outlet_profile, drag_lift_id) plus precision, pattern, rho_out, device
    and stream (a cudaStream_t handle as int).
    """

    def __init__(self, mesh, uavg=0.05, vavg=0.0, rho_ini=1.0, viscosity=0.01,
                 inlet_profile=2, collision_model=BGKW, curved_boundaries=2, outlet_profile=2,
                 drag_lift_id=0, precision=FP64, pattern=AB, rho_out=1.0, device=0, stream=None,
                 tile_variant=0):
        L = self.L = load()
        p = make_params(uavg, vavg, rho_ini, viscosity, inlet_profile, collision_model,
                        curved_boundaries, outlet_profile, drag_lift_id, precision, pattern,
                        rho_out, device, stream, tile_variant)
        precision, pattern = p.precision, p.pattern
        self.mesh = mesh
        self.h = C.c_void_p()
        _check(L.lbm_create(C.byref(mesh.c_struct()), C.byref(p), C.byref(self.h)), "lbm_create")
        n, m = C.c_int32(), C.c_int32()
        _check(L.lbm_get_dims(self.h, C.byref(n), C.byref(m)), "lbm_get_dims")
        self.n, self.m = n.value, m.value
        self.N = self.n * self.m
        self.precision, self.pattern = precision, pattern

    def set_state(self, f=None, rho=None, u=None, v=None):
        arrs = [None if a is None else np.ascontiguousarray(a, np.float64) for a in (f, rho, u, v)]
        _check(self.L.lbm_set_state(self.h, *[_ptr(a) for a in arrs]), "lbm_set_state")

    def step(self, nsteps, check_every=0):
        rows = nsteps // check_every if check_every > 0 else 0
        res = np.zeros((max(rows, 1), 4))
        _check(self.L.lbm_step(self.h, int(nsteps), int(check_every), _ptr(res) if rows else None),
               "lbm_step")
        return res[:rows]

    def fields(self, f=False, metaf=False):
        out = {k: np.zeros(self.N) for k in ("rho", "u", "v")}
        if f:
            out["f"] = np.zeros((self.N, 9))
        if metaf:
            out["metaf"] = np.zeros((self.N, 9))
        _check(self.L.lbm_get_fields(self.h, _ptr(out["rho"]), _ptr(out["u"]), _ptr(out["v"]),
                                     _ptr(out.get("f")), _ptr(out.get("metaf"))),
               "lbm_get_fields")
        return out

    def check(self):
        d = lbm_diagnostics()
        _check(self.L.lbm_check(self.h, C.byref(d)), "lbm_check")
        return {"iteration": d.iteration, "l2_full": d.l2_full, "du_rel": d.du_rel,
                "mass": d.mass, "momentum": tuple(d.momentum), "force": tuple(d.force),
                "max_speed": d.max_speed}

    def autotune(self, steps_per_trial=10, cache_path=None):
        """Pick the fastest fused-step tile for this domain (before set_state)."""
        buf = C.create_string_buffer(1024)
        _check(self.L.lbm_autotune(self.h, int(steps_per_trial),
                                   None if cache_path is None else str(cache_path).encode(),
                                   buf, len(buf)), "lbm_autotune")
        import json
        return json.loads(buf.value.decode())

    def info(self):
        it, db, bpn = C.c_int64(), C.c_int64(), C.c_int32()
        _check(self.L.lbm_get_info(self.h, C.byref(it), C.byref(db), C.byref(bpn)), "lbm_get_info")
        return {"iteration": it.value, "device_bytes": db.value, "bytes_per_node_step": bpn.value}

    def close(self):
        if getattr(self, "h", None):
            self.L.lbm_destroy(self.h)
            self.h = None

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class Batch:
    """Many independent domains stepped together (wraps lbm_batch).

    ``cases`` is a list of (Mesh, params dict); all cases share precision
    (fp64, fp32 or fp16dev), the A-B pattern and the collision model.
    """

    def __init__(self, cases, precision=FP32, device=0):
        L = self.L = load()
        if isinstance(precision, str):
            precision = PRECISIONS[precision]
        self.meshes = [m for m, _ in cases]
        self._mesh_structs = (lbm_mesh * len(cases))(*[m.c_struct() for m in self.meshes])
        self._params = (lbm_params * len(cases))(
            *[make_params(precision=precision, pattern=AB, device=device, **p) for _, p in cases])
        self.h = C.c_void_p()
        _check(L.lbm_batch_create(self._mesh_structs, self._params, len(cases), C.byref(self.h)),
               "lbm_batch_create")
        self.n_cases = len(cases)

    def autotune(self, steps_per_trial=5):
        import json
        buf = C.create_string_buffer(512)
        _check(self.L.lbm_batch_autotune(self.h, int(steps_per_trial), buf, len(buf)),
               "lbm_batch_autotune")
        return json.loads(buf.value.decode())

    def set_rest(self):
        _check(self.L.lbm_batch_set_rest(self.h), "lbm_batch_set_rest")

    def set_state(self, case, rho, u, v):
        arrs = [np.ascontiguousarray(a, np.float64) for a in (rho, u, v)]
        _check(self.L.lbm_batch_set_state(self.h, int(case), *[_ptr(a) for a in arrs]),
               "lbm_batch_set_state")

    def set_tile(self, variant):
        _check(self.L.lbm_batch_set_tile(self.h, int(variant)), "lbm_batch_set_tile")

    def set_launch(self, special_blocks_per_sm=0, bulk_prefetch=False):
        _check(self.L.lbm_batch_set_launch(self.h, int(special_blocks_per_sm), int(bulk_prefetch)),
               "lbm_batch_set_launch")

    def run(self, max_steps, check_every=100, tol=1e-6, raise_on_nan=True):
        nc = self.n_cases
        steps = np.zeros(nc, np.int64)
        du = np.zeros(nc)
        conv = np.zeros(nc, np.int32)
        sec = C.c_double()
        st = self.L.lbm_batch_run(self.h, int(max_steps), int(check_every), float(tol), _ptr(steps),
                                  _ptr(du), _ptr(conv), C.byref(sec))
        if st != LBM_DIVERGED or raise_on_nan:
            _check(st, "lbm_batch_run")
        return {"steps": steps, "du_rel": du, "converged": conv, "seconds": sec.value}

    def fields(self, case):
        n, m = C.c_int32(), C.c_int32()
        _check(self.L.lbm_batch_dims(self.h, int(case), C.byref(n), C.byref(m)), "lbm_batch_dims")
        N = n.value * m.value
        out = {k: np.zeros(N) for k in ("rho", "u", "v")}
        _check(self.L.lbm_batch_get_fields(self.h, int(case), _ptr(out["rho"]), _ptr(out["u"]),
                                           _ptr(out["v"])), "lbm_batch_get_fields")
        return out

    def info(self):
        nodes, fluid, dev = C.c_int64(), C.c_int64(), C.c_int64()
        var = C.c_int32()
        _check(self.L.lbm_batch_info(self.h, C.byref(nodes), C.byref(fluid), C.byref(var),
                                     C.byref(dev)), "lbm_batch_info")
        return {"nodes": nodes.value, "fluid_nodes": fluid.value, "tile_variant": var.value,
                "device_bytes": dev.value}

    def close(self):
        if getattr(self, "h", None):
            self.L.lbm_batch_destroy(self.h)
            self.h = None

    __del__ = close


class lbm_sg_config(C.Structure):
    _fields_ = [("height", C.c_int32), ("width", C.c_int32), ("in_channels", C.c_int32),
                ("out_channels", C.c_int32), ("base", C.c_int32), ("max_batch", C.c_int32),
                ("lr", C.c_float), ("beta1", C.c_float), ("beta2", C.c_float), ("eps", C.c_float),
                ("seed", C.c_uint64), ("device", C.c_int32), ("weight_decay", C.c_float),
                ("coarse_weight", C.c_float), ("coarse_block", C.c_int32),
                ("products", C.c_int32)]


def _load_sg(L):
    vp, i32, dp = C.c_void_p, C.c_int32, C.c_void_p
    if getattr(L, "_sg_ready", False):
        return L
    L.lbm_sg_create.argtypes = [C.POINTER(lbm_sg_config), C.POINTER(vp)]
    L.lbm_sg_destroy.argtypes = [vp]
    L.lbm_sg_destroy.restype = None
    L.lbm_sg_num_params.argtypes = [vp, C.POINTER(C.c_int64)]
    L.lbm_sg_get_params.argtypes = [vp, dp]
    L.lbm_sg_set_params.argtypes = [vp, dp]
    L.lbm_sg_forward.argtypes = [vp, i32, dp, dp]
    L.lbm_sg_loss_grads.argtypes = [vp, i32, dp, dp, dp, C.POINTER(C.c_double), dp]
    L.lbm_sg_adam_step.argtypes = [vp]
    L.lbm_sg_set_lr.argtypes = [vp, C.c_float]
    L.lbm_sg_set_dataset.argtypes = [vp, i32, dp, dp, dp]
    L.lbm_sg_train.argtypes = [vp, i32, dp, i32, C.POINTER(C.c_double)]
    for n in ("lbm_sg_create", "lbm_sg_num_params", "lbm_sg_get_params", "lbm_sg_set_params",
              "lbm_sg_forward", "lbm_sg_loss_grads", "lbm_sg_adam_step", "lbm_sg_set_dataset",
              "lbm_sg_train", "lbm_sg_set_lr"):
        getattr(L, n).restype = C.c_int
    L._sg_ready = True
    return L


# tensor-core paths of the network's products (lbm_sg_config.products)
PRODUCTS = {"tcgen05": 0, "mma": 1, "tcgen05-gather": 2, "tcgen05-1seg": 3}


class Surrogate:
    """The warm-start network (wraps lbm_sg): NHWC float32 arrays on the host."""

    def __init__(self, height=256, width=256, in_channels=4, out_channels=3, base=32,
                 max_batch=8, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8, seed=0, device=0,
                 weight_decay=0.0, coarse_weight=0.0, coarse_block=8, products="tcgen05"):
        """products: "tcgen05" (the convolution products on the 5th-generation
        tensor cores where the shapes allow, the TMA-fed halo-tile form for
        3x3 layers with W a multiple of 128 and C a multiple of 32, four row
        segments per convolution block where H is a multiple of 4),
        "tcgen05-1seg" (the same with one row segment per convolution block),
        "tcgen05-gather" (tcgen05 with the im2col gather only) or "mma" (every
        product on the mma.sync kernels)."""
        L = self.L = _load_sg(load())
        if products not in PRODUCTS:
            raise ValueError("products must be one of " + ", ".join(PRODUCTS))
        self.cfg = lbm_sg_config(height, width, in_channels, out_channels, base, max_batch, lr,
                                 beta1, beta2, eps, seed, device, weight_decay, coarse_weight,
                                 coarse_block, PRODUCTS[products])
        self.h = C.c_void_p()
        _check(L.lbm_sg_create(C.byref(self.cfg), C.byref(self.h)), "lbm_sg_create")
        n = C.c_int64()
        _check(L.lbm_sg_num_params(self.h, C.byref(n)), "lbm_sg_num_params")
        self.num_params = n.value

    def params(self):
        out = np.zeros(self.num_params, np.float32)
        _check(self.L.lbm_sg_get_params(self.h, _ptr(out)), "lbm_sg_get_params")
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.num_params
        _check(self.L.lbm_sg_set_params(self.h, _ptr(p)), "lbm_sg_set_params")

    def forward(self, x):
        x = np.ascontiguousarray(x, np.float32)
        B = x.shape[0]
        c = self.cfg
        y = np.zeros((B, c.height, c.width, c.out_channels), np.float32)
        for i in range(0, B, c.max_batch):
            xb = np.ascontiguousarray(x[i:i + c.max_batch])
            yb = np.zeros((len(xb), c.height, c.width, c.out_channels), np.float32)
            _check(self.L.lbm_sg_forward(self.h, len(xb), _ptr(xb), _ptr(yb)), "lbm_sg_forward")
            y[i:i + len(xb)] = yb
        return y

    def loss_grads(self, x, t, m=None):
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        m = None if m is None else np.ascontiguousarray(m, np.float32)
        loss = C.c_double()
        g = np.zeros(self.num_params, np.float32)
        _check(self.L.lbm_sg_loss_grads(self.h, x.shape[0], _ptr(x), _ptr(t), _ptr(m),
                                        C.byref(loss), _ptr(g)), "lbm_sg_loss_grads")
        return loss.value, g

    def adam_step(self):
        _check(self.L.lbm_sg_adam_step(self.h), "lbm_sg_adam_step")

    def set_lr(self, lr):
        _check(self.L.lbm_sg_set_lr(self.h, float(lr)), "lbm_sg_set_lr")

    def set_dataset(self, x, y, m):
        self._ds = [np.ascontiguousarray(a, np.float32) for a in (x, y, m)]
        _check(self.L.lbm_sg_set_dataset(self.h, len(x), *[_ptr(a) for a in self._ds]),
               "lbm_sg_set_dataset")

    def train(self, order, batch):
        order = np.ascontiguousarray(order, np.int32)
        loss = C.c_double()
        _check(self.L.lbm_sg_train(self.h, int(batch), _ptr(order), len(order), C.byref(loss)),
               "lbm_sg_train")
        return loss.value

    def close(self):
        if getattr(self, "h", None):
            self.L.lbm_sg_destroy(self.h)
            self.h = None

    __del__ = close
