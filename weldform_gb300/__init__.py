"""weldform_gb300 — GB300 (sm_103a) kick-drift SPH solid step behind WeldForm's Domain API.

The compute path is the in-tree CUDA library ``_build/libweldform_gb300.so``
(C ABI declared in ``include/weldform_gb300.h``).  This module is a thin
ctypes mirror of the reference's ``SPH::Domain`` members (Source/Domain.h:113-537)
so a WeldForm driver translates line for line:

    dom = Domain()                                   # Domain::Domain
    dom.Kernel_Set(0)                                # Domain::Kernel_Set(Qubic_Spline)
    dom.AddCylinderLength(1, (0, 0, 0), R, L, dx / 2, rho, h, False)
    dom.AssignZone((-1, -1, -1), (1, 1, 2 * dx), 2)
    ...
    dom.SolveDiffUpdateKickDrift(tf, dt, dtOut)

There is no CPU fallback: importing works without a GPU, but creating a
``Domain`` fails loudly when the library or a CUDA device is missing.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional, Sequence

import numpy as np

__all__ = ["Domain", "WFError", "load_library", "LIB_PATH", "PRECISION_FP64", "PRECISION_MIXED",
           "BILINEAR", "HOLLOMON", "JOHNSON_COOK", "CONTACT_WANG", "CONTACT_PENALTY", "CONTACT_AREA", "PARAMS"]

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libweldform_gb300.so")

PRECISION_FP64 = 0
PRECISION_MIXED = 1
BILINEAR, HOLLOMON, JOHNSON_COOK = 0, 1, 2
CONTACT_WANG, CONTACT_PENALTY, CONTACT_AREA = 0, 1, 2
# Parameters of the reaction-force adjoint, in the order of its gradient.
PARAMS = ("E", "sy0", "Ep", "A", "B", "n", "C", "m", "mu", "PFAC")

_ERRNAMES = {1: "WF_ERR_ARG", 2: "WF_ERR_CUDA", 3: "WF_ERR_NAN", 4: "WF_ERR_NBR_OVERFLOW", 5: "WF_ERR_TIMEOUT",
             6: "WF_ERR_STATE", 7: "WF_ERR_NOMEM", 8: "WF_ERR_UNSUPPORTED"}

TENSOR_FIELDS = ("Sigma", "ShearStress", "StrainRate", "RotationRate", "Strain", "Strain_pl", "Strain_pl_incr", "TIR", "gradCorrM")
VECTOR_FIELDS = ("x", "v", "a", "Displacement", "normal", "contforce")


class WFError(RuntimeError):
    """A non-zero status from the C ABI; ``code`` is the WF_ERR_* value."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"{_ERRNAMES.get(code, code)}: {msg}")
        self.code = code


_D = ctypes.c_double
_I = ctypes.c_int
_I64 = ctypes.c_int64
_P = ctypes.c_void_p
_S = ctypes.c_char_p
_DP = ctypes.POINTER(ctypes.c_double)
_IP = ctypes.POINTER(ctypes.c_int32)
_I64P = ctypes.POINTER(ctypes.c_int64)

# name -> argtypes (return type is int for all)
_SIGS = {
    "domain_create": [_I, ctypes.POINTER(_P)],
    "domain_destroy": [_P],
    "set_domain_f64": [_P, _S, _D],
    "set_domain_i32": [_P, _S, _I],
    "get_domain_f64": [_P, _S, _DP],
    "get_domain_i32": [_P, _S, _I64P],
    "kernel_set": [_P, _I],
    "add_box_length": [_P, _I, _DP, _D, _D, _D, _D, _D, _D, _I, _I, _I, _I],
    "add_cylinder_length": [_P, _I, _DP, _D, _D, _D, _D, _D, _I, _I],
    "assign_zone": [_P, _DP, _DP, _I, _I64P],
    "set_particle_f64": [_P, _S, _I, _D],
    "set_particle_i32": [_P, _S, _I, _I],
    "set_particle_array_f64": [_P, _S, _DP, _I64],
    "get_particle_array_f64": [_P, _S, _DP, _I64],
    "get_particle_array_f64_async": [_P, _S, _DP, _I64],
    "get_particle_array_i32": [_P, _S, _IP, _I64],
    "set_particle_array_i32": [_P, _S, _IP, _I64],
    "add_material": [_P, _I, _DP, _I, ctypes.POINTER(_I)],
    "add_amplitude": [_P, _I, _DP, _DP, _I],
    "add_velocity_bc": [_P, _I, _DP, _DP, _I, _I, _D],
    "add_rigid_plane": [_P, _I, _I, _DP, _DP, _I, _D, _I, ctypes.POINTER(_I)],
    "set_mesh_velocity": [_P, _I, _DP, _DP],
    "get_contact_force": [_P, _I, _DP],
    "solve_kickdrift": [_P, _D, _D, _D, _I64],
    "solve_leapfrog": [_P, _D, _D, _D, _I64],
    "prepare_kickdrift": [_P, _D],
    "step": [_P, _I64],
    "neighbour_search": [_P],
    "get_neighbours": [_P, _I64P, _IP, _I64],
    "get_contact_pairs": [_P, _I64P, _IP, _I64],
    "synchronize": [_P],
    "step_timed": [_P, _I64, _DP, _I64P],
    "checkpoint_save": [_P, _I],
    "checkpoint_restore": [_P, _I],
    "checkpoint_free": [_P, _I],
    "autotune": [_P, _I, ctypes.POINTER(_I)],
    "profile_steps": [_P, _I64, ctypes.c_char_p, _I, _DP, _I64P, _I, ctypes.POINTER(_I)],
    "adjoint_reaction_loss": [_P, _I64, _I, _I, _I, _DP, _I64, _I, _DP, _DP, _DP, _DP, _DP],
    "batch_specimens": [_P, _I64P, _I64P, _I],
    "batch_get_i32": [_P, _I, _S, _I64P],
}
EXPORTS = ["version", "last_error"] + list(_SIGS)


def bind(lib: ctypes.CDLL, prefix: str):
    """Attach argument types for every entry point of a library with this ABI."""
    for name, args in _SIGS.items():
        fn = getattr(lib, prefix + name)
        fn.argtypes = args
        fn.restype = ctypes.c_int
    getattr(lib, prefix + "last_error").restype = ctypes.c_char_p
    getattr(lib, prefix + "version").restype = ctypes.c_int
    return lib


_lib: Optional[ctypes.CDLL] = None


def load_library(path: str = LIB_PATH) -> ctypes.CDLL:
    """Load the in-tree CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is None or path != LIB_PATH:
        if not os.path.exists(path):
            raise OSError(f"weldform_gb300 CUDA library not built: {path} (run __graft_entry__.build())")
        lib = bind(ctypes.CDLL(path), "wf_")
        if path != LIB_PATH:
            return lib
        _lib = lib
    return _lib


def _v3(v) -> ctypes.Array:
    a = (ctypes.c_double * 3)()
    for k in range(3):
        a[k] = float(v[k])
    return a


class Domain:
    """Mirror of ``SPH::Domain`` for the kick-drift solid path.

    ``lib``/``prefix`` select the implementation behind the C ABI; the default
    is this package's CUDA library.
    """

    def __init__(self, dimension: int = 3, lib: Optional[ctypes.CDLL] = None, prefix: str = "wf_"):
        self._lib = lib if lib is not None else load_library()
        self._px = prefix
        self._h = ctypes.c_void_p()
        self._call("domain_create", int(dimension), ctypes.byref(self._h))
        self.Dimension = dimension

    # ------------------------------------------------------------ plumbing
    def _fn(self, name):
        return getattr(self._lib, self._px + name)

    def _call(self, name, *args):
        rc = self._fn(name)(*args)
        if rc != 0:
            msg = self._fn("last_error")().decode(errors="replace")
            raise WFError(rc, msg)
        return rc

    def close(self):
        if self._h and self._h.value:
            self._fn("domain_destroy")(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ------------------------------------------------------------ scalars
    def set(self, name: str, value):
        if isinstance(value, (bool, int, np.integer)) and not isinstance(value, float):
            self._call("set_domain_i32", self._h, name.encode(), int(value))
        else:
            self._call("set_domain_f64", self._h, name.encode(), float(value))

    def set_f64(self, name: str, value: float):
        self._call("set_domain_f64", self._h, name.encode(), float(value))

    def get(self, name: str) -> float:
        out = ctypes.c_double()
        self._call("get_domain_f64", self._h, name.encode(), ctypes.byref(out))
        return out.value

    def geti(self, name: str) -> int:
        out = ctypes.c_int64()
        self._call("get_domain_i32", self._h, name.encode(), ctypes.byref(out))
        return out.value

    @property
    def particle_count(self) -> int:
        return self.geti("particle_count")

    @property
    def Time(self) -> float:
        return self.get("Time")

    # ------------------------------------------------------------ reference API
    def Kernel_Set(self, kernel_type: int = 0):
        self._call("kernel_set", self._h, int(kernel_type))

    def AddBoxLength(self, tag: int, V: Sequence[float], Lx: float, Ly: float, Lz: float, r: float, Density: float,
                     h: float, type: int = 1, rotation: int = 0, random: bool = False, Fixed: bool = False):
        self._call("add_box_length", self._h, int(tag), _v3(V), Lx, Ly, Lz, r, Density, h, int(type), int(rotation),
                   int(bool(random)), int(bool(Fixed)))

    def AddCylinderLength(self, tag: int, V: Sequence[float], Rxy: float, Lz: float, r: float, Density: float,
                          h: float, Fixed: bool = False, ghost: bool = False):
        self._call("add_cylinder_length", self._h, int(tag), _v3(V), Rxy, Lz, r, Density, h, int(bool(Fixed)),
                   int(bool(ghost)))

    def AssignZone(self, start: Sequence[float], end: Sequence[float], id: int) -> int:
        c = ctypes.c_int64()
        self._call("assign_zone", self._h, _v3(start), _v3(end), int(id), ctypes.byref(c))
        return c.value

    def set_particles(self, field: str, value, zone: int = -1):
        """Assign a per-particle public field (Particle.h:50-265) for a zone (or all)."""
        if isinstance(value, (bool, int, np.integer)) and not isinstance(value, float) and field in (
                "PresEq", "Fail", "Material_model", "mat", "Material", "ID", "IsFree", "print_history", "Thermal_BC"):
            self._call("set_particle_i32", self._h, field.encode(), int(zone), int(value))
        else:
            self._call("set_particle_f64", self._h, field.encode(), int(zone), float(value))

    def add_material(self, model: int, params: Sequence[float]) -> int:
        arr = (ctypes.c_double * len(params))(*[float(p) for p in params])
        out = ctypes.c_int()
        self._call("add_material", self._h, int(model), arr, len(params), ctypes.byref(out))
        return out.value

    def add_amplitude(self, id: int, time: Sequence[float], value: Sequence[float]):
        t = (ctypes.c_double * len(time))(*time)
        v = (ctypes.c_double * len(value))(*value)
        self._call("add_amplitude", self._h, int(id), t, v, len(time))

    def add_velocity_bc(self, zone: int, value: Sequence[float], value_ang: Sequence[float] = (0, 0, 0),
                        value_type: int = 0, amp_id: int = 0, amp_factor: float = 1.0):
        self._call("add_velocity_bc", self._h, int(zone), _v3(value), _v3(value_ang), int(value_type), int(amp_id),
                   float(amp_factor))

    def add_rigid_plane(self, axis: int, positaxisorent: bool, p1: Sequence[float], p2: Sequence[float], dens: int,
                        zone_id: int, hfac: float = 1.1) -> int:
        out = ctypes.c_int()
        self._call("add_rigid_plane", self._h, int(axis), int(bool(positaxisorent)), _v3(p1), _v3(p2), int(dens),
                   float(hfac), int(zone_id), ctypes.byref(out))
        return out.value

    def set_mesh_velocity(self, mesh: int, v: Sequence[float], w: Sequence[float] = (0, 0, 0)):
        self._call("set_mesh_velocity", self._h, int(mesh), _v3(v), _v3(w))

    def contact_force(self, mesh: int = 0) -> np.ndarray:
        out = (ctypes.c_double * 3)()
        self._call("get_contact_force", self._h, int(mesh), out)
        return np.array(out[:])

    def prepare(self, dt: float):
        self._call("prepare_kickdrift", self._h, float(dt))

    def step(self, n: int = 1):
        self._call("step", self._h, int(n))

    def SolveDiffUpdateKickDrift(self, tf: float, dt: float, dtOut: float, TheFileKey=None, maxidx: int = 1000000):
        self._call("solve_kickdrift", self._h, float(tf), float(dt), float(dtOut), int(maxidx))

    def SolveDiffUpdateLeapFrog(self, tf: float, dt: float, dtOut: float, TheFileKey=None, maxidx: int = 1000000):
        self._call("solve_leapfrog", self._h, float(tf), float(dt), float(dtOut), int(maxidx))

    def neighbour_search(self):
        self._call("neighbour_search", self._h)

    def synchronize(self):
        self._call("synchronize", self._h)

    def checkpoint_save(self, slot: int = 0):
        self._call("checkpoint_save", self._h, int(slot))

    def checkpoint_restore(self, slot: int = 0):
        self._call("checkpoint_restore", self._h, int(slot))

    def checkpoint_free(self, slot: int = 0):
        self._call("checkpoint_free", self._h, int(slot))

    def autotune(self, steps: int = 5) -> int:
        """Pick the mixed gathers' block size and lanes per particle by
        timing every pair; returns the block size (the lanes are the domain
        field "gather_lanes")."""
        b = ctypes.c_int()
        self._call("autotune", self._h, int(steps), ctypes.byref(b))
        return b.value

    def step_timed(self, n: int):
        """n steps between CUDA events on the domain's stream: (ms, kernel launches)."""
        ms = ctypes.c_double()
        nl = ctypes.c_int64()
        self._call("step_timed", self._h, int(n), ctypes.byref(ms), ctypes.byref(nl))
        return ms.value, nl.value

    def profile_steps(self, n: int, cap: int = 64):
        """Per-kernel event timing over n instrumented steps: {name: (total_ms, launches)}."""
        L = 48
        names = ctypes.create_string_buffer(cap * L)
        tot = (ctypes.c_double * cap)()
        cnt = (ctypes.c_int64 * cap)()
        nk = ctypes.c_int()
        self._call("profile_steps", self._h, int(n), names, L, tot, cnt, cap, ctypes.byref(nk))
        out = {}
        for k in range(nk.value):
            nm = names.raw[k * L:(k + 1) * L].split(b"\0", 1)[0].decode()
            out[nm] = (tot[k], int(cnt[k]))
        return out

    def adjoint_reaction_loss(self, steps: int, every: int, target, mesh: int = 0, axis: int = 2,
                              checkpoint_every: int = 20):
        """Loss (1/S) sum_s (F_s - target_s)^2 of the mesh's reaction force
        sampled every `every` steps, and its gradient with respect to PARAMS by
        the reverse-mode adjoint (plain FP64 form, checkpoint every
        `checkpoint_every` steps).  Returns a dict with loss, grad (PARAMS
        order), curve (the sampled F_s), fwd_ms and adj_ms; the domain ends
        `steps` steps later."""
        t = np.ascontiguousarray(target, dtype=np.float64).ravel()
        loss = ctypes.c_double()
        grad = np.zeros(len(PARAMS))
        curve = np.zeros(t.size)
        fms, ams = ctypes.c_double(), ctypes.c_double()
        self._call("adjoint_reaction_loss", self._h, int(steps), int(every), int(mesh), int(axis),
                   t.ctypes.data_as(_DP), t.size, int(checkpoint_every), ctypes.byref(loss),
                   grad.ctypes.data_as(_DP), curve.ctypes.data_as(_DP), ctypes.byref(fms), ctypes.byref(ams))
        return {"loss": loss.value, "grad": grad, "curve": curve, "fwd_ms": fms.value, "adj_ms": ams.value}

    # ------------------------------------------------------------ arrays
    def get_array(self, field: str, out: np.ndarray = None) -> np.ndarray:
        """Particle field in original particle order.  ``out`` (optional) is a
        C-contiguous array of the field's dtype and size (e.g. pinned host
        memory) that receives the values; it is returned as given."""
        n = self.particle_count
        i32 = field in ("ID", "Nb", "IsFree", "Thermal_BC")
        comps = 1 if i32 else (9 if field in TENSOR_FIELDS else (3 if field in VECTOR_FIELDS else 1))
        dt = np.int32 if i32 else np.float64
        if out is None:
            buf = np.empty(n * comps, dtype=dt)
        else:
            if out.dtype != dt or out.size != n * comps or not out.flags["C_CONTIGUOUS"]:
                raise ValueError(f"{field}: out must be a C-contiguous {np.dtype(dt).name} array of {n * comps} values")
            buf = out.reshape(-1)
        if i32:
            self._call("get_particle_array_i32", self._h, field.encode(), buf.ctypes.data_as(_IP), buf.size)
        else:
            self._call("get_particle_array_f64", self._h, field.encode(), buf.ctypes.data_as(_DP), buf.size)
        if out is not None:
            return out
        return buf.reshape(n, comps) if comps > 1 else buf

    def get_array_async(self, field: str, out: np.ndarray) -> np.ndarray:
        """Enqueues a read of a float particle field into ``out`` (C-contiguous
        float64 of the field's size; pinned host memory lets the copy overlap
        later steps) and returns it at once; it holds the values after
        ``synchronize()`` (wf_get_particle_array_f64_async)."""
        n = self.particle_count
        comps = 9 if field in TENSOR_FIELDS else (3 if field in VECTOR_FIELDS else 1)
        if out.dtype != np.float64 or out.size != n * comps or not out.flags["C_CONTIGUOUS"]:
            raise ValueError(f"{field}: out must be a C-contiguous float64 array of {n * comps} values")
        buf = out.reshape(-1)
        self._call("get_particle_array_f64_async", self._h, field.encode(), buf.ctypes.data_as(_DP), buf.size)
        return out

    def set_array(self, field: str, values):
        if field in ("ID", "mat", "Material_model", "Fail", "Material", "not_write_surf_ID", "Thermal_BC"):
            a = np.ascontiguousarray(values, dtype=np.int32).ravel()
            self._call("set_particle_array_i32", self._h, field.encode(), a.ctypes.data_as(_IP), a.size)
            return
        a = np.ascontiguousarray(values, dtype=np.float64).ravel()
        self._call("set_particle_array_f64", self._h, field.encode(), a.ctypes.data_as(_DP), a.size)

    # ------------------------------------------------------------ batches
    def batch_specimens(self, ranges):
        """Specimens as [first, last) ranges of original particle indices,
        each with its own rebuild schedule (wf_batch_specimens)."""
        first = np.array([a for a, _ in ranges], dtype=np.int64)
        count = np.array([b - a for a, b in ranges], dtype=np.int64)
        self._call("batch_specimens", self._h, first.ctypes.data_as(_I64P), count.ctypes.data_as(_I64P), len(ranges))

    def batch_get(self, spec: int, name: str) -> int:
        v = ctypes.c_int64()
        self._call("batch_get_i32", self._h, int(spec), name.encode(), ctypes.byref(v))
        return int(v.value)

    def _rows(self, which: str):
        n = self.particle_count
        off = np.zeros(n + 1, dtype=np.int64)
        self._call(which, self._h, off.ctypes.data_as(_I64P), None, 0)
        idx = np.zeros(max(int(off[-1]), 1), dtype=np.int32)
        self._call(which, self._h, off.ctypes.data_as(_I64P), idx.ctypes.data_as(_IP), idx.size)
        return off, idx[: int(off[-1])]

    def neighbours(self):
        """SMPairs as CSR (offsets, indices) in original order, canonical row order."""
        return self._rows("get_neighbours")

    def contact_pairs(self):
        return self._rows("get_contact_pairs")
