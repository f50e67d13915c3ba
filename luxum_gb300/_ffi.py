"""ctypes view of the C ABI declared in include/luxum.h.

The engine is the in-tree libluxum.so (CUDA kernels for sm_103a).  Loading fails loudly
when it has not been built: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import pathlib

PKG = pathlib.Path(__file__).resolve().parent
LIB_PATH = PKG / "libluxum.so"

LX_OK, LX_ERR_INVALID, LX_ERR_UNSUPPORTED, LX_ERR_CUDA, LX_ERR_OOM, LX_ERR_BLOWUP, LX_ERR_IO, LX_ERR_STATE = range(8)
LX_PREC_FP64, LX_PREC_FP32, LX_PREC_FP16S = 0, 1, 2
LX_REQ_QUEUED, LX_REQ_RUNNING, LX_REQ_DONE, LX_REQ_FAILED, LX_REQ_CANCELLED = 0, 1, 2, 3, 4
LX_CPML_REFERENCE, LX_CPML_STANDARD = 0, 1
LX_SRC_CW_HARD, LX_SRC_PULSE_SOFT = 0, 1
EX, EY, EZ, HX, HY, HZ, ETOTAL = range(7)
COMPONENTS = ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz", "Etotal")
STATUS_NAMES = {0: "LX_OK", 1: "LX_ERR_INVALID", 2: "LX_ERR_UNSUPPORTED", 3: "LX_ERR_CUDA", 4: "LX_ERR_OOM",
                5: "LX_ERR_BLOWUP", 6: "LX_ERR_IO", 7: "LX_ERR_STATE"}


class Params(C.Structure):
    """lx_params: the public members of Luxum's reader class plus engine options."""

    _fields_ = [
        ("isPlanar", C.c_int),
        ("Nx", C.c_int), ("Ny", C.c_int), ("Nz", C.c_int),
        ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double),
        ("S", C.c_double),
        ("num_timesteps", C.c_int),
        ("npX", C.c_int), ("npY", C.c_int), ("n_threads", C.c_int),
        ("usePS", C.c_int),
        ("Nx_source", C.c_int), ("Ny_source", C.c_int), ("Nz_source", C.c_int),
        ("amp_source", C.c_double), ("omega_source", C.c_double),
        ("usePW", C.c_int),
        ("kx_pw", C.c_double), ("ky_pw", C.c_double), ("kz_pw", C.c_double),
        ("Ex_pw", C.c_double), ("Ey_pw", C.c_double), ("Ez_pw", C.c_double),
        ("off_pw", C.c_double),
        ("x1_pw", C.c_int), ("y1_pw", C.c_int), ("z1_pw", C.c_int),
        ("x2_pw", C.c_int), ("y2_pw", C.c_int), ("z2_pw", C.c_int),
        ("usePML", C.c_int),
        ("d_pml", C.c_double), ("sigma", C.c_double), ("sigma_m", C.c_double),
        ("kappa", C.c_double), ("a_max", C.c_double), ("a_m", C.c_double),
        ("precision", C.c_int),
        ("pw_sigma", C.c_double),
        ("cpml_mode", C.c_int),
        ("source_kind", C.c_int),
        ("src_t0", C.c_double), ("src_tw", C.c_double),
        ("monitor_every", C.c_int),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class Info(C.Structure):
    _fields_ = [("cells", C.c_size_t), ("device_bytes", C.c_size_t), ("psi_h_entries", C.c_size_t),
                ("psi_e_entries", C.c_size_t), ("slab", C.c_int * 3), ("uniform", C.c_int), ("field_bytes", C.c_int)]


class TuneEntry(C.Structure):
    _fields_ = [("planar", C.c_int), ("size_class", C.c_int), ("precision", C.c_int), ("slab_class", C.c_int),
                ("march", C.c_int)]


class ServerConfig(C.Structure):
    _fields_ = [("precision", C.c_int), ("chunk", C.c_int), ("budget_bytes", C.c_double), ("max_running", C.c_int),
                ("tune_steps", C.c_int), ("tune_table", C.POINTER(TuneEntry)), ("tune_entries", C.c_int)]


class Request(C.Structure):
    _fields_ = [("params", Params), ("steps", C.c_int), ("material", C.POINTER(C.c_double) * 3),
                ("material_scale", C.c_double), ("n_boxes", C.c_int), ("boxes", C.POINTER(C.c_int)),
                ("box_eps", C.POINTER(C.c_double)), ("dft_axis", C.c_int), ("dft_index", C.c_int),
                ("dft_every", C.c_int), ("nfreq", C.c_int), ("omega", C.POINTER(C.c_double))]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_longlong), ("queued", C.c_longlong), ("running", C.c_longlong),
                ("done", C.c_longlong), ("failed", C.c_longlong), ("cancelled", C.c_longlong),
                ("bytes_running", C.c_double), ("peak_bytes_running", C.c_double), ("peak_running", C.c_int),
                ("cell_updates", C.c_double), ("busy_seconds", C.c_double), ("chunks", C.c_longlong),
                ("tune_seconds", C.c_double), ("tuned_classes", C.c_int), ("enqueue_seconds", C.c_double),
                ("prepare_seconds", C.c_double), ("wait_seconds", C.c_double), ("join_seconds", C.c_double),
                ("retire_seconds", C.c_double)]


SNAPSHOT_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_int))

_lib = None


def _proto(lib, name, restype, *argtypes):
    f = getattr(lib, name)
    f.restype = restype
    f.argtypes = list(argtypes)


def declare(lib) -> None:
    """Attaches the prototypes of include/luxum.h to a loaded library."""
    P = C.POINTER
    sim = C.c_void_p
    _proto(lib, "lx_params_init", None, P(Params))
    _proto(lib, "lx_params_from_yaml", C.c_int, C.c_char_p, P(Params))
    _proto(lib, "lx_sim_create", C.c_int, P(Params), P(C.c_void_p))
    _proto(lib, "lx_sim_destroy", None, sim)
    _proto(lib, "lx_params_device_bytes", C.c_int, P(Params), P(C.c_size_t))
    _proto(lib, "lx_params_step_bytes", C.c_int, P(Params), P(C.c_double))
    _proto(lib, "lx_sim_reset", C.c_int, sim)
    _proto(lib, "lx_sim_set_cb", C.c_int, sim, C.c_int, P(C.c_double), C.c_size_t)
    _proto(lib, "lx_sim_set_material", C.c_int, sim, C.c_int, P(C.c_double), C.c_size_t, C.c_double)
    _proto(lib, "lx_sim_set_eps_box", C.c_int, sim, P(C.c_int), P(C.c_int), C.c_double)
    _proto(lib, "lx_sim_step", C.c_int, sim, C.c_int)
    _proto(lib, "lx_sim_sync", C.c_int, sim)
    _proto(lib, "lx_sim_field_shape", C.c_int, sim, C.c_int, P(C.c_int))
    _proto(lib, "lx_sim_read_field", C.c_int, sim, C.c_int, P(C.c_double), C.c_size_t)
    _proto(lib, "lx_sim_write_field", C.c_int, sim, C.c_int, P(C.c_double), C.c_size_t)
    _proto(lib, "lx_sim_read_field_noalloc", C.c_int, sim, C.c_int, P(C.c_double), C.c_size_t)
    _proto(lib, "lx_sim_timestep", C.c_int, sim)
    _proto(lib, "lx_sim_max_e2", C.c_int, sim, P(C.c_double))
    _proto(lib, "lx_sim_set_probes", C.c_int, sim, P(C.c_int), C.c_int, C.c_int)
    _proto(lib, "lx_sim_read_probes", C.c_int, sim, P(C.c_double), C.c_size_t, P(C.c_int))
    _proto(lib, "lx_sim_add_dft_plane", C.c_int, sim, C.c_int, C.c_int, C.c_int, P(C.c_double), C.c_int, P(C.c_int))
    _proto(lib, "lx_sim_read_dft", C.c_int, sim, C.c_int, P(C.c_double), C.c_size_t)
    _proto(lib, "lx_sim_save", C.c_int, sim, C.c_char_p)
    _proto(lib, "lx_sim_set_max_series", C.c_int, sim, C.c_int)
    _proto(lib, "lx_sim_read_max_series", C.c_int, sim, P(C.c_int), P(C.c_double), C.c_int, P(C.c_int))
    _proto(lib, "lx_sim_load", C.c_int, sim, C.c_char_p)
    _proto(lib, "lx_sim_dft_flux", C.c_int, sim, C.c_int, P(C.c_double), C.c_int)
    _proto(lib, "lx_sim_set_snapshots", C.c_int, sim, C.c_int, C.c_uint, SNAPSHOT_FN, C.c_void_p)
    _proto(lib, "lx_sim_set_hdf5_output", C.c_int, sim, C.c_int, C.c_int, C.c_int, C.c_char_p)
    _proto(lib, "lx_sim_set_stream", C.c_int, sim, C.c_void_p)
    _proto(lib, "lx_sim_time_kernels", C.c_int, sim, C.c_int, P(C.c_double))
    _proto(lib, "lx_sim_info", C.c_int, sim, P(Info))
    _proto(lib, "lx_sim_counters", C.c_int, sim, P(C.c_uint64), P(C.c_uint64), P(C.c_uint64))
    _proto(lib, "lx_hdf5_write", C.c_int, C.c_char_p, C.c_int, P(C.c_char_p), P(P(C.c_double)), P(C.c_int))
    _proto(lib, "lx_hdf5_read", C.c_int, C.c_char_p, C.c_char_p, P(C.c_double), C.c_size_t, P(C.c_int))
    _proto(lib, "lx_batch_create", C.c_int, P(C.c_void_p))
    _proto(lib, "lx_batch_destroy", None, C.c_void_p)
    _proto(lib, "lx_batch_add", C.c_int, C.c_void_p, sim)
    _proto(lib, "lx_batch_remove", C.c_int, C.c_void_p, sim)
    _proto(lib, "lx_batch_size", C.c_int, C.c_void_p)
    _proto(lib, "lx_batch_set_chunk", C.c_int, C.c_void_p, C.c_int)
    _proto(lib, "lx_batch_step", C.c_int, C.c_void_p, C.c_int)
    _proto(lib, "lx_batch_step_async", C.c_int, C.c_void_p, C.c_int)
    _proto(lib, "lx_batch_wait", C.c_int, C.c_void_p)
    _proto(lib, "lx_batch_set_march", C.c_int, C.c_void_p, C.c_int, C.c_int)
    _proto(lib, "lx_batch_get_march", C.c_int, C.c_void_p, P(C.c_int), P(C.c_int))
    _proto(lib, "lx_batch_autotune", C.c_int, C.c_void_p, C.c_int, P(C.c_int), P(C.c_int))
    _proto(lib, "lx_sim_tune_class", C.c_int, C.c_void_p, P(TuneEntry))
    _proto(lib, "lx_batch_set_tune_table", C.c_int, C.c_void_p, P(TuneEntry), C.c_int)
    _proto(lib, "lx_batch_get_tune_table", C.c_int, C.c_void_p, P(TuneEntry), C.c_int, P(C.c_int))
    _proto(lib, "lx_batch_tune_member", C.c_int, C.c_void_p, C.c_void_p, C.c_int, P(C.c_int))
    srv, ll = C.c_void_p, C.c_longlong
    _proto(lib, "lx_params_field_shape", C.c_int, P(Params), C.c_int, P(C.c_int))
    _proto(lib, "lx_server_config_init", None, P(ServerConfig))
    _proto(lib, "lx_request_init", None, P(Request))
    _proto(lib, "lx_server_create", C.c_int, P(ServerConfig), P(C.c_void_p))
    _proto(lib, "lx_server_destroy", None, srv)
    _proto(lib, "lx_server_submit", C.c_int, srv, P(Request), P(ll))
    _proto(lib, "lx_server_poll", C.c_int, srv, ll, P(C.c_int))
    _proto(lib, "lx_server_wait", C.c_int, srv, ll, C.c_double, P(C.c_int))
    _proto(lib, "lx_server_cancel", C.c_int, srv, ll)
    _proto(lib, "lx_server_flux", C.c_int, srv, ll, P(C.c_double), C.c_int)
    _proto(lib, "lx_server_max_e2", C.c_int, srv, ll, P(C.c_double))
    _proto(lib, "lx_server_times", C.c_int, srv, ll, P(C.c_double))
    _proto(lib, "lx_server_take", C.c_int, srv, ll, P(C.c_void_p))
    _proto(lib, "lx_server_release", C.c_int, srv, ll)
    _proto(lib, "lx_server_error", C.c_char_p, srv, ll)
    _proto(lib, "lx_server_stats_get", C.c_int, srv, P(ServerStats))
    _proto(lib, "lx_server_tune_table", C.c_int, srv, P(TuneEntry), C.c_int, P(C.c_int))
    _proto(lib, "lx_host_alloc", C.c_int, C.c_size_t, P(C.c_void_p))
    _proto(lib, "lx_host_free", None, C.c_void_p)
    _proto(lib, "lx_trim_device_memory", C.c_int)
    _proto(lib, "lx_last_error", C.c_char_p, sim)
    _proto(lib, "lx_version", C.c_char_p)


def lib():
    """The loaded engine library (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: build the engine first (python -c 'import __graft_entry__ as g; g.build()')")
        handle = C.CDLL(str(LIB_PATH))
        declare(handle)
        _lib = handle
    return _lib


class LuxumError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status
