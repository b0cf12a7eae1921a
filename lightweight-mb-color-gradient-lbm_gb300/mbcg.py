"""Python face of the mbcg C ABI (include/mbcg.h): parameter presets and a ctypes binding.

The solver itself is the CUDA library ``libmbcg.so`` built next to this file from ``csrc/``;
every call below goes through its ``extern "C"`` entry points.  There is no CPU fallback:
``Library()`` raises if the shared object is missing or fails to load.

Case presets follow the reference's cases (``jet/``, ``bubble/``, ``rti/``) and the
workloads the solver is benchmarked on; sizes are lattice sizes including the one-node ghost
frame of the reference's layout (``utilities/indexing.cuh:10-14``), so a box of
``L`` fluid nodes per axis is ``L + 2`` nodes.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmbcg.so")

NFIELDS = 11
FIELD_NAMES = ("rhor", "rhob", "ux", "uy", "uz", "Pixx", "Pixy", "Piyy", "Piyz", "Pizz", "Pixz")

BC_PERIODIC, BC_INOUT, BC_WALL = 0, 1, 2
OUTLET_CONVECTIVE, OUTLET_ZERO_GRADIENT = 0, 1
FP32, FP16, BF16 = 0, 1, 2
IC_JET, IC_BUBBLE, IC_RTI, IC_NONE = 0, 1, 2, 3
VTI_ASCII, VTI_RAW = 0, 1
VTI_REFERENCE_FIELDS = 0x1F


class Params(ctypes.Structure):
    """Mirror of ``mbcg_params`` (include/mbcg.h)."""

    _fields_ = [
        ("q", ctypes.c_int32),
        ("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32),
        ("bc", ctypes.c_int32 * 3),
        ("outlet", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("ic", ctypes.c_int32),
        ("tau", ctypes.c_double),
        ("sigma", ctypes.c_double),
        ("beta", ctypes.c_double),
        ("rho_r0", ctypes.c_double), ("rho_b0", ctypes.c_double),
        ("gravity", ctypes.c_double * 3),
        ("jet_radius", ctypes.c_double),
        ("jet_velocity", ctypes.c_double),
        ("jet_center", ctypes.c_double * 2),
        ("jet_phase", ctypes.c_double),
        ("inlet_noise", ctypes.c_double),
        ("seed", ctypes.c_uint64),
        ("bubble_radius", ctypes.c_double),
        ("bubble_center", ctypes.c_double * 3),
        ("bubble_width", ctypes.c_double),
        ("bubble_phase", ctypes.c_double),
        ("rti_position", ctypes.c_double),
        ("rti_amplitude", ctypes.c_double),
        ("rti_width", ctypes.c_double),
        ("rti_phase_above", ctypes.c_double),
        ("rti_mode", ctypes.c_int32 * 2),
        ("omega2_conservative", ctypes.c_int32),
        ("wait_test_cycles", ctypes.c_int32),
        ("rho_scale", ctypes.c_double),
        ("u_ref", ctypes.c_double),
        ("pi_scale", ctypes.c_double),
        ("tau_b", ctypes.c_double),
    ]

    @property
    def shape(self):
        """(nz, ny, nx): numpy shape of one field in the dense reference layout."""
        return (self.nz, self.ny, self.nx)

    def active_nodes(self) -> int:
        return (self.nx - 2) * (self.ny - 2) * (self.nz - 2)

    def copy(self) -> "Params":
        p = Params()
        ctypes.pointer(p)[0] = self
        return p

    def describe(self) -> dict:
        d = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            d[name] = list(v) if hasattr(v, "__len__") else v
        return d


def default_params() -> Params:
    """The reference's shipped constants (constants.cuh:9-93): D3Q27 128^3 jet along y."""
    p = Params()
    p.q = 27
    p.nx = p.ny = p.nz = 128
    p.bc[0], p.bc[1], p.bc[2] = BC_PERIODIC, BC_INOUT, BC_PERIODIC
    p.outlet = OUTLET_CONVECTIVE
    p.precision = FP32
    p.ic = IC_JET
    p.tau = 1.0
    p.sigma = 0.1
    p.beta = 0.9
    p.rho_r0 = p.rho_b0 = 1.0
    p.jet_radius = 12.0
    p.jet_velocity = 0.05
    p.jet_center[0] = (p.nx - 1) / 2.0
    p.jet_center[1] = (p.nz - 1) / 2.0
    p.jet_phase = -1.0
    p.inlet_noise = 0.0
    p.seed = 12345
    p.bubble_radius = 30.0
    p.bubble_center[0] = (p.nx - 1) / 2.0
    p.bubble_center[1] = (p.ny - 1) / 2.0
    p.bubble_center[2] = (p.nz - 1) / 2.0
    p.bubble_width = 0.0
    p.bubble_phase = -1.0
    p.rti_position = (p.ny - 1) / 2.0
    p.rti_amplitude = 4.0
    p.rti_width = 4.0
    p.rti_phase_above = -1.0
    p.rti_mode[0] = p.rti_mode[1] = 1
    p.rho_scale = 0.01
    p.u_ref = 0.05
    p.pi_scale = 0.05 * 0.05
    return p


def reference_jet_params(nx: int, ny: int, nz: int, q: int = 27, tau: float = 1.0, sigma: float = 0.1,
                         beta: float = 0.9, radius: float = 12.0, velocity: float = 0.05) -> Params:
    """The reference's own jet case (jet along y, periodic x/z, convective outlet, blue jet)
    on an nx*ny*nz lattice, with the constants it is compiled with (constants.cuh)."""
    p = default_params()
    p.q = q
    p.nx, p.ny, p.nz = nx, ny, nz
    p.tau, p.sigma, p.beta = tau, sigma, beta
    p.jet_radius, p.jet_velocity = radius, velocity
    p.jet_center[0] = (nx - 1) / 2.0
    p.jet_center[1] = (nz - 1) / 2.0
    p.bubble_center[0] = (nx - 1) / 2.0
    p.bubble_center[1] = (ny - 1) / 2.0
    p.bubble_center[2] = (nz - 1) / 2.0
    p.rti_position = (ny - 1) / 2.0
    return p


def bubble_params(L: int = 64, q: int = 19, radius: Optional[float] = None, width: float = 3.0,
                  tau: float = 0.8, sigma: float = 0.01, beta: float = 0.7, precision: int = FP32,
                  conservative: bool = False) -> Params:
    """Static-bubble Laplace case: L^3 fluid nodes, fully periodic, phi = +1 (red) inside a
    sphere of radius L/4 centred in the box, tanh profile of the given width, rho = 1."""
    p = default_params()
    p.q = q
    p.nx = p.ny = p.nz = L + 2
    p.bc[0] = p.bc[1] = p.bc[2] = BC_PERIODIC
    p.ic = IC_BUBBLE
    p.tau, p.sigma, p.beta = tau, sigma, beta
    p.bubble_radius = L / 4.0 if radius is None else radius
    # fluid node i sits at lattice index i + 1: the centre of fluid nodes 0..L-1 is L/2 + 0.5
    c = L / 2.0 + 0.5
    p.bubble_center[0] = p.bubble_center[1] = p.bubble_center[2] = c
    p.bubble_width = width
    p.bubble_phase = 1.0
    p.precision = precision
    p.omega2_conservative = 1 if conservative else 0
    return p


def rti_params(L: int = 128, H: Optional[int] = None, q: int = 27, ratio: float = 3.0, g: float = 1e-5,
               tau: float = 0.55, sigma: float = 5e-4, beta: float = 0.7, amplitude: Optional[float] = None,
               precision: int = FP32) -> Params:
    """Rayleigh-Taylor case: L x L fluid nodes periodic in x/y, walls on the z ghost layers
    z = 0 and z = H - 1 (H = 4L lattice planes), heavy red phase (phi = +1, density
    ratio `ratio`) above z = H/2 + A cos(2 pi x / L) cos(2 pi y / L), gravity along -z."""
    p = default_params()
    H = 4 * L if H is None else H
    p.q = q
    p.nx = p.ny = L + 2
    p.nz = H
    p.bc[0] = p.bc[1] = BC_PERIODIC
    p.bc[2] = BC_WALL
    p.ic = IC_RTI
    p.tau, p.sigma, p.beta = tau, sigma, beta
    p.rho_r0, p.rho_b0 = ratio, 1.0
    p.gravity[0], p.gravity[1], p.gravity[2] = 0.0, 0.0, -g
    p.rti_position = H / 2.0
    p.rti_amplitude = (0.05 * L) if amplitude is None else amplitude
    p.rti_width = 4.0
    p.rti_phase_above = 1.0
    p.rti_mode[0] = p.rti_mode[1] = 1
    p.precision = precision
    return p


def jet_params(nx: int = 256, ny: int = 256, nz: int = 1024, q: int = 27, diameter: float = 32.0,
               velocity: float = 0.05, noise: float = 0.01, tau: float = 0.51, sigma: float = 1e-3,
               beta: float = 0.7, seed: int = 12345, precision: int = FP32) -> Params:
    """Liquid-jet case: nx x ny fluid nodes periodic in x/y; inlet ghost plane z = 0 with a
    disc of the given diameter injecting red fluid (phi = +1) at u_z = velocity plus
    +-noise*velocity uniform per-node noise on all components each step; zero-gradient
    outflow on the ghost plane z = nz + 1; nz fluid planes."""
    p = default_params()
    p.q = q
    p.nx, p.ny, p.nz = nx + 2, ny + 2, nz + 2
    p.bc[0] = p.bc[1] = BC_PERIODIC
    p.bc[2] = BC_INOUT
    p.outlet = OUTLET_ZERO_GRADIENT
    p.ic = IC_JET
    p.tau, p.sigma, p.beta = tau, sigma, beta
    p.jet_radius = diameter / 2.0
    p.jet_velocity = velocity
    p.jet_center[0] = (p.nx - 1) / 2.0
    p.jet_center[1] = (p.ny - 1) / 2.0
    p.jet_phase = 1.0
    p.inlet_noise = noise
    p.seed = seed
    p.u_ref = velocity
    p.pi_scale = velocity * velocity
    p.precision = precision
    return p


# ----------------------------------------------------------------------------- ctypes ABI
class Moments(ctypes.Structure):
    """Mirror of ``mbcg_moments``."""
    _fields_ = [("f", ctypes.c_void_p * NFIELDS), ("pitch", ctypes.c_int64),
                ("precision", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class Diag(ctypes.Structure):
    """Mirror of ``mbcg_diag``."""
    _fields_ = [("mass_r", ctypes.c_double), ("mass_b", ctypes.c_double),
                ("momentum", ctypes.c_double * 3), ("p_in", ctypes.c_double),
                ("p_out", ctypes.c_double), ("dp", ctypes.c_double),
                ("nonfinite", ctypes.c_int64), ("nodes", ctypes.c_int64)]

    def as_dict(self) -> dict:
        return {"mass_r": self.mass_r, "mass_b": self.mass_b, "momentum": list(self.momentum),
                "p_in": self.p_in, "p_out": self.p_out, "dp": self.dp,
                "nonfinite": self.nonfinite, "nodes": self.nodes}


class PhaseStats(ctypes.Structure):
    """Mirror of ``mbcg_phase_stats``."""
    _fields_ = [("volume_tracked", ctypes.c_double), ("volume_other", ctypes.c_double),
                ("interface_area", ctypes.c_double), ("interface_nodes", ctypes.c_int64),
                ("penetration", ctypes.c_double), ("centroid", ctypes.c_double * 3),
                ("components", ctypes.c_int64), ("largest_component", ctypes.c_int64),
                ("detached", ctypes.c_int64), ("detached_volume", ctypes.c_int64),
                ("status", ctypes.c_int32), ("reserved", ctypes.c_int32)]

    def as_dict(self) -> dict:
        d = {n: getattr(self, n) for n, _ in self._fields_ if n != "reserved"}
        d["centroid"] = list(self.centroid)
        return d


STATS_COMPONENTS = 1


class ServerConfig(ctypes.Structure):
    """Mirror of ``mbcg_server_config``."""
    _fields_ = [("arena_bytes", ctypes.c_int64), ("max_live", ctypes.c_int32), ("chunk_steps", ctypes.c_int32),
                ("keep_results", ctypes.c_int32), ("backfill", ctypes.c_int32), ("zchunk", ctypes.c_int32),
                ("calibrate", ctypes.c_int32), ("policy", ctypes.c_int32), ("fill_waves", ctypes.c_int32)]


POLICY_FIFO, POLICY_SJF = 0, 1
REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_FAILED = 0, 1, 2, 3


class RequestInfo(ctypes.Structure):
    """Mirror of ``mbcg_request_info``."""
    _fields_ = [("id", ctypes.c_int64), ("state", ctypes.c_int32), ("status", ctypes.c_int32),
                ("steps", ctypes.c_int64), ("steps_done", ctypes.c_int64), ("t_submit", ctypes.c_double),
                ("t_admit", ctypes.c_double), ("t_done", ctypes.c_double), ("state_hash", ctypes.c_uint64),
                ("diag", Diag)]

    def as_dict(self) -> dict:
        return {"id": self.id, "state": self.state, "status": self.status, "steps": self.steps,
                "steps_done": self.steps_done, "t_submit": self.t_submit, "t_admit": self.t_admit,
                "t_done": self.t_done, "state_hash": self.state_hash, "diag": self.diag.as_dict()}


class ServerStats(ctypes.Structure):
    """Mirror of ``mbcg_server_stats``."""
    _fields_ = [("submitted", ctypes.c_int64), ("completed", ctypes.c_int64), ("failed", ctypes.c_int64),
                ("live", ctypes.c_int64), ("queued", ctypes.c_int64), ("node_updates", ctypes.c_int64),
                ("compositions", ctypes.c_int64), ("replays", ctypes.c_int64), ("arena_bytes", ctypes.c_int64),
                ("arena_peak_bytes", ctypes.c_int64), ("zchunk", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("plane_ns", ctypes.c_double * 10), ("tile_overhead_planes", ctypes.c_double),
                ("busy_s", ctypes.c_double)]

    BODIES = ("q19_f32", "q19_f16", "q19_bf16", "q27_f32", "q27_f16", "q27_bf16",
              "q19_f32_periodic", "q19_f16_periodic", "q27_f32_periodic", "q27_f16_periodic")

    def as_dict(self) -> dict:
        d = {n: getattr(self, n) for n, _ in self._fields_ if n not in ("plane_ns", "reserved")}
        d["plane_ns"] = dict(zip(self.BODIES, list(self.plane_ns)))
        return d


class MbcgError(RuntimeError):
    pass


_P = ctypes.POINTER
_VP = ctypes.c_void_p

_PROTOS = {
    "mbcg_params_default": (None, [_P(Params)]),
    "mbcg_create": (ctypes.c_int, [_P(Params), _P(_VP)]),
    "mbcg_destroy": (ctypes.c_int, [_VP]),
    "mbcg_init": (ctypes.c_int, [_VP, _VP]),
    "mbcg_step": (ctypes.c_int, [_VP, ctypes.c_int32, _VP]),
    "mbcg_rcs": (ctypes.c_int, [_VP, _VP]),
    "mbcg_bc": (ctypes.c_int, [_VP, _VP]),
    "mbcg_swap": (ctypes.c_int, [_VP]),
    "mbcg_fields": (ctypes.c_int, [_VP, _P(Moments), _P(Moments)]),
    "mbcg_steps_done": (ctypes.c_int64, [_VP]),
    "mbcg_copy_out": (ctypes.c_int, [_VP, _VP * NFIELDS, _VP]),
    "mbcg_copy_in": (ctypes.c_int, [_VP, _VP * NFIELDS, _VP]),
    "mbcg_run_host": (ctypes.c_int, [_VP, ctypes.c_int32, _P(_VP), _P(_VP), ctypes.c_int32, _VP]),
    "mbcg_diagnostics": (ctypes.c_int, [_VP, _P(Diag), _VP]),
    "mbcg_status": (ctypes.c_int, [_VP, _P(ctypes.c_int32)]),
    "mbcg_case_params": (ctypes.c_int, [_VP, _P(Params)]),
    "mbcg_phase_statistics": (ctypes.c_int, [_VP, ctypes.c_int32, _P(PhaseStats), _VP]),
    "mbcg_write_vti": (ctypes.c_int, [_VP, ctypes.c_char_p, ctypes.c_uint32, ctypes.c_int32, _VP]),
    "mbcg_writer_create": (ctypes.c_int, [ctypes.c_int32, _P(_VP)]),
    "mbcg_writer_snapshot": (ctypes.c_int, [_VP, _VP, ctypes.c_char_p, ctypes.c_uint32, ctypes.c_int32, _VP]),
    "mbcg_writer_flush": (ctypes.c_int, [_VP]),
    "mbcg_writer_destroy": (ctypes.c_int, [_VP]),
    "mbcg_checkpoint_save": (ctypes.c_int, [_VP, ctypes.c_char_p, _VP]),
    "mbcg_checkpoint_load": (ctypes.c_int, [ctypes.c_char_p, _P(_VP)]),
    "mbcg_get_shape": (ctypes.c_int, [_VP, _P(ctypes.c_int32), _P(ctypes.c_int32)]),
    "mbcg_set_shape": (ctypes.c_int, [_VP, ctypes.c_int32, ctypes.c_int32]),
    "mbcg_autotune": (ctypes.c_int, [_VP, ctypes.c_int32, _P(ctypes.c_double), _VP]),
    "mbcg_rcs_moments": (ctypes.c_int, [_P(Params), _P(Moments), _P(Moments), ctypes.c_int64, _VP]),
    "mbcg_bc_moments": (ctypes.c_int, [_P(Params), _P(Moments), _P(Moments), ctypes.c_int64, _VP]),
    "mbcg_init_moments": (ctypes.c_int, [_P(Params), _P(Moments), _VP]),
    "mbcg_active_nodes": (ctypes.c_int64, [_P(Params)]),
    "mbcg_diagnostics_static": (ctypes.c_int, [_P(Params), _P(Moments), _P(Diag), _VP]),
    "mbcg_launches_per_step": (ctypes.c_int32, [_VP]),
    "mbcg_server_config_default": (None, [_P(ServerConfig)]),
    "mbcg_server_create": (ctypes.c_int, [_P(ServerConfig), _P(_VP)]),
    "mbcg_server_destroy": (ctypes.c_int, [_VP]),
    "mbcg_server_submit": (ctypes.c_int, [_VP, _P(Params), ctypes.c_int64, _P(ctypes.c_int64)]),
    "mbcg_server_poll": (ctypes.c_int, [_VP, ctypes.c_int64, _P(RequestInfo)]),
    "mbcg_server_wait": (ctypes.c_int, [_VP, ctypes.c_int64, ctypes.c_double, _P(RequestInfo)]),
    "mbcg_server_drain": (ctypes.c_int, [_VP, ctypes.c_double]),
    "mbcg_server_fetch": (ctypes.c_int, [_VP, ctypes.c_int64, _VP * NFIELDS]),
    "mbcg_server_release": (ctypes.c_int, [_VP, ctypes.c_int64]),
    "mbcg_server_get_stats": (ctypes.c_int, [_VP, _P(ServerStats)]),
    "mbcg_last_error": (ctypes.c_char_p, []),
    "mbcg_version": (ctypes.c_char_p, []),
}


class Library:
    """ctypes handle on libmbcg.so; raises if the CUDA library is absent."""

    _instance = None

    def __init__(self, path: str = LIB_PATH):
        if not os.path.exists(path):
            raise MbcgError(f"CUDA library not built: {path} (run __graft_entry__.build())")
        self.path = path
        self.lib = ctypes.CDLL(path)
        for name, (res, args) in _PROTOS.items():
            fn = getattr(self.lib, name)
            fn.restype = res
            fn.argtypes = args

    @classmethod
    def get(cls) -> "Library":
        if cls._instance is None:
            cls._instance = Library()
        return cls._instance

    def check(self, rc: int, what: str) -> None:
        if rc != 0:
            msg = self.lib.mbcg_last_error()
            raise MbcgError(f"{what} failed ({rc}): {msg.decode() if msg else ''}")

    def __getattr__(self, name):
        return getattr(self.lib, name)


def _stream_ptr(stream) -> Optional[int]:
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return int(stream.cuda_stream)  # torch.cuda.Stream


class Case:
    """Library-owned simulation state (mbcg_case*)."""

    def __init__(self, params: Params, lib: Optional[Library] = None, _handle=None):
        self.lib = lib or Library.get()
        self.params = params.copy()
        if _handle is not None:
            self.handle = _handle
            return
        h = ctypes.c_void_p()
        self.lib.check(self.lib.mbcg_create(ctypes.byref(self.params), ctypes.byref(h)), "mbcg_create")
        self.handle = h

    @classmethod
    def from_checkpoint(cls, path: str, lib: Optional[Library] = None) -> "Case":
        """A case restored from mbcg_checkpoint_save's file: parameters, step count, state."""
        lib = lib or Library.get()
        h = ctypes.c_void_p()
        lib.check(lib.mbcg_checkpoint_load(os.fsencode(path), ctypes.byref(h)), "mbcg_checkpoint_load")
        p = Params()
        lib.check(lib.mbcg_case_params(h, ctypes.byref(p)), "mbcg_case_params")
        return cls(p, lib, _handle=h)

    def checkpoint(self, path: str, stream=None):
        self.lib.check(self.lib.mbcg_checkpoint_save(self.handle, os.fsencode(path), _stream_ptr(stream)),
                       "mbcg_checkpoint_save")

    def phase_statistics(self, components: bool = False, stream=None) -> dict:
        """In-situ phase statistics of state A (volumes, interface area, penetration, regions)."""
        st = PhaseStats()
        self.lib.check(self.lib.mbcg_phase_statistics(self.handle, STATS_COMPONENTS if components else 0,
                                                      ctypes.byref(st), _stream_ptr(stream)),
                       "mbcg_phase_statistics")
        return st.as_dict()

    def write_vti(self, path: str, fields: int = 0, fmt: int = VTI_ASCII, stream=None):
        """State A as a VTI image (fields: bit mask over the 11 fields, 0 = the reference's five)."""
        self.lib.check(self.lib.mbcg_write_vti(self.handle, os.fsencode(path), int(fields), int(fmt),
                                               _stream_ptr(stream)), "mbcg_write_vti")

    def close(self):
        if getattr(self, "handle", None):
            self.lib.mbcg_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def init(self, stream=None):
        self.lib.check(self.lib.mbcg_init(self.handle, _stream_ptr(stream)), "mbcg_init")

    def step(self, n: int = 1, stream=None):
        self.lib.check(self.lib.mbcg_step(self.handle, int(n), _stream_ptr(stream)), "mbcg_step")

    def rcs(self, stream=None):
        self.lib.check(self.lib.mbcg_rcs(self.handle, _stream_ptr(stream)), "mbcg_rcs")

    def bc(self, stream=None):
        self.lib.check(self.lib.mbcg_bc(self.handle, _stream_ptr(stream)), "mbcg_bc")

    def swap(self):
        self.lib.check(self.lib.mbcg_swap(self.handle), "mbcg_swap")

    @property
    def steps_done(self) -> int:
        return int(self.lib.mbcg_steps_done(self.handle))

    def fields(self):
        a, b = Moments(), Moments()
        self.lib.check(self.lib.mbcg_fields(self.handle, ctypes.byref(a), ctypes.byref(b)), "mbcg_fields")
        return a, b

    def copy_out(self, stream=None, out: Optional[np.ndarray] = None) -> np.ndarray:
        """State A as an (11, nz, ny, nx) float32 array in the reference's dense layout."""
        p = self.params
        if out is None:
            out = np.empty((NFIELDS,) + p.shape, dtype=np.float32)
        ptrs = (_VP * NFIELDS)(*[out[f].ctypes.data for f in range(NFIELDS)])
        self.lib.check(self.lib.mbcg_copy_out(self.handle, ptrs, _stream_ptr(stream)), "mbcg_copy_out")
        return out

    def copy_in(self, state: np.ndarray, stream=None):
        state = np.ascontiguousarray(state, dtype=np.float32)
        ptrs = (_VP * NFIELDS)(*[state[f].ctypes.data for f in range(NFIELDS)])
        self.lib.check(self.lib.mbcg_copy_in(self.handle, ptrs, _stream_ptr(stream)), "mbcg_copy_in")

    def run_host(self, states: Sequence[np.ndarray], outs: Sequence[np.ndarray], nsteps: int = 1, stream=None):
        """mbcg_run_host: for each j, copy_in(states[j]); step(nsteps); copy_out(outs[j]), with the
        transfers of consecutive states overlapped (pinned host arrays, e.g. from
        torch.empty(..., pin_memory=True).numpy(), let both link directions run at once)."""
        if len(states) != len(outs):
            raise ValueError("one output per input state")
        keep = []
        pin, pout = [], []
        for a, o in zip(states, outs):
            a = np.ascontiguousarray(a, dtype=np.float32)
            if o.dtype != np.float32 or not o.flags.c_contiguous or o.shape != (NFIELDS,) + self.params.shape:
                raise ValueError("outputs must be C-contiguous float32 arrays of the state's shape")
            keep.append(a)
            pin.extend(a[f].ctypes.data for f in range(NFIELDS))
            pout.extend(o[f].ctypes.data for f in range(NFIELDS))
        n = len(states)
        cin = (_VP * max(1, len(pin)))(*pin)
        cout = (_VP * max(1, len(pout)))(*pout)
        self.lib.check(self.lib.mbcg_run_host(self.handle, n, ctypes.cast(cin, _P(_VP)), ctypes.cast(cout, _P(_VP)),
                                              nsteps, _stream_ptr(stream)), "mbcg_run_host")

    def diagnostics(self, stream=None) -> dict:
        d = Diag()
        self.lib.check(self.lib.mbcg_diagnostics(self.handle, ctypes.byref(d), _stream_ptr(stream)),
                       "mbcg_diagnostics")
        return d.as_dict()

    def status(self) -> int:
        s = ctypes.c_int32(0)
        self.lib.check(self.lib.mbcg_status(self.handle, ctypes.byref(s)), "mbcg_status")
        return int(s.value)

    def launches_per_step(self) -> int:
        return int(self.lib.mbcg_launches_per_step(self.handle))

    @property
    def shape(self) -> tuple:
        """(block_rows, zchunk) of the step launches."""
        w, z = ctypes.c_int32(0), ctypes.c_int32(0)
        self.lib.check(self.lib.mbcg_get_shape(self.handle, ctypes.byref(w), ctypes.byref(z)), "mbcg_get_shape")
        return int(w.value), int(z.value)

    def set_shape(self, block_rows: int, zchunk: int):
        self.lib.check(self.lib.mbcg_set_shape(self.handle, int(block_rows), int(zchunk)), "mbcg_set_shape")

    def autotune(self, repeats: int = 3, stream=None) -> float:
        """Measure the candidate launch shapes on this case and keep the fastest; returns ms/step."""
        ms = ctypes.c_double(0.0)
        self.lib.check(self.lib.mbcg_autotune(self.handle, int(repeats), ctypes.byref(ms), _stream_ptr(stream)),
                       "mbcg_autotune")
        return float(ms.value)


class Writer:
    """Asynchronous VTI writer (mbcg_writer*): snapshots are taken on the case's stream and written
    to disk while the case keeps stepping."""

    def __init__(self, max_pending: int = 2, lib: Optional[Library] = None):
        self.lib = lib or Library.get()
        h = ctypes.c_void_p()
        self.lib.check(self.lib.mbcg_writer_create(int(max_pending), ctypes.byref(h)), "mbcg_writer_create")
        self.handle = h

    def snapshot(self, case: Case, path: str, fields: int = 0, fmt: int = VTI_RAW, stream=None):
        self.lib.check(self.lib.mbcg_writer_snapshot(self.handle, case.handle, os.fsencode(path), int(fields),
                                                     int(fmt), _stream_ptr(stream)), "mbcg_writer_snapshot")

    def flush(self):
        self.lib.check(self.lib.mbcg_writer_flush(self.handle), "mbcg_writer_flush")

    def close(self):
        if getattr(self, "handle", None):
            rc = self.lib.mbcg_writer_destroy(self.handle)
            self.handle = None
            self.lib.check(rc, "mbcg_writer_destroy")

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def read_vti(path: str) -> dict:
    """Fields of a VTI image written by mbcg_write_vti / Writer (ASCII or appended raw) as float32
    arrays of shape (nz, ny, nx), keyed by name."""
    import re
    data = open(path, "rb").read()
    head_end = data.find(b"<AppendedData")
    text = data[: head_end if head_end >= 0 else len(data)].decode()
    ext = [int(v) for v in re.search(r'WholeExtent="([^"]+)"', text).group(1).split()]
    shape = (ext[5] + 1, ext[3] + 1, ext[1] + 1)
    out = {}
    if head_end >= 0:
        start = data.index(b"_", head_end) + 1
        for name, off in re.findall(r'Name="(\w+)" format="appended" offset="(\d+)"', text):
            o = start + int(off)
            nbytes = int(np.frombuffer(data[o:o + 8], dtype=np.uint64)[0])
            out[name] = np.frombuffer(data[o + 8:o + 8 + nbytes], dtype=np.float32).reshape(shape)
    else:
        for name, body in re.findall(r'Name="(\w+)" format="ascii">\n(.*?)</DataArray>', text, flags=re.S):
            out[name] = np.array(body.split(), dtype=np.float32).reshape(shape)
    return out


def server_config(**kw) -> ServerConfig:
    """mbcg_server_config with the library defaults, then the given fields."""
    cfg = ServerConfig()
    Library.get().mbcg_server_config_default(ctypes.byref(cfg))
    for k, v in kw.items():
        setattr(cfg, k, v)
    return cfg


class Server:
    """Continuous-batching server (mbcg_server*): many cases resident on one GPU, advanced
    together by the persistent batch kernel."""

    def __init__(self, config: Optional[ServerConfig] = None, lib: Optional[Library] = None, **kw):
        self.lib = lib or Library.get()
        cfg = config if config is not None else server_config(**kw)
        h = ctypes.c_void_p()
        self.lib.check(self.lib.mbcg_server_create(ctypes.byref(cfg), ctypes.byref(h)), "mbcg_server_create")
        self.handle = h

    def close(self):
        if getattr(self, "handle", None):
            self.lib.mbcg_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def submit(self, params: Params, nsteps: int) -> int:
        rid = ctypes.c_int64(0)
        p = params.copy()
        self.lib.check(self.lib.mbcg_server_submit(self.handle, ctypes.byref(p), int(nsteps), ctypes.byref(rid)),
                       "mbcg_server_submit")
        return int(rid.value)

    def poll(self, rid: int) -> RequestInfo:
        info = RequestInfo()
        self.lib.check(self.lib.mbcg_server_poll(self.handle, int(rid), ctypes.byref(info)), "mbcg_server_poll")
        return info

    def wait(self, rid: int, timeout: float = 600.0) -> RequestInfo:
        info = RequestInfo()
        self.lib.check(self.lib.mbcg_server_wait(self.handle, int(rid), float(timeout), ctypes.byref(info)),
                       "mbcg_server_wait")
        return info

    def drain(self, timeout: float = 3600.0):
        self.lib.check(self.lib.mbcg_server_drain(self.handle, float(timeout)), "mbcg_server_drain")

    def fetch(self, rid: int, shape) -> np.ndarray:
        """Final state of a finished request (keep_results) as (11, nz, ny, nx) float32."""
        out = np.empty((NFIELDS,) + tuple(shape), dtype=np.float32)
        ptrs = (_VP * NFIELDS)(*[out[f].ctypes.data for f in range(NFIELDS)])
        self.lib.check(self.lib.mbcg_server_fetch(self.handle, int(rid), ptrs), "mbcg_server_fetch")
        return out

    def release(self, rid: int):
        self.lib.check(self.lib.mbcg_server_release(self.handle, int(rid)), "mbcg_server_release")

    def stats(self) -> ServerStats:
        st = ServerStats()
        self.lib.check(self.lib.mbcg_server_get_stats(self.handle, ctypes.byref(st)), "mbcg_server_get_stats")
        return st


def moments_from_tensors(tensors: Sequence, pitch: int, precision: int = FP32) -> Moments:
    """mbcg_moments view over 11 device tensors (torch) in the reference layout."""
    m = Moments()
    for f in range(NFIELDS):
        m.f[f] = tensors[f].data_ptr()
    m.pitch = pitch
    m.precision = precision
    return m
