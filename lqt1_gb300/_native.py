"""ctypes binding of the native library (lqt1_gb300/_lib/liblqt.so, include/lqt.h).

There is no fallback: if the library is missing or the GPU is unusable every
call raises.  The compute path is the CUDA code behind the C ABI.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "liblqt.so")

OK, ERR_INVALID, ERR_CUDA, ERR_NUMERIC, ERR_TIMEOUT, ERR_NOMEM, ERR_STATE, ERR_IO = range(8)
LVEPI, LVENDO, EPI, ENDO, MCELL, EMPTY = 0, 1, 2, 3, 4, 255
FP64, MIXED = 0, 1
NSTATE = 40
PRESET = {"baseline": 0, "default": 1, "con": 2, "lqt1": 3, "gpu3d": 4, "gpu2d": 5}


class LqtError(RuntimeError):
    def __init__(self, code: int, where: str, msg: str):
        super().__init__(f"{where}: status {code}: {msg}")
        self.code = code


class Model(C.Structure):
    _fields_ = [("dss_shift", C.c_double), ("fss_shift", C.c_double), ("pca_scale", C.c_double),
                ("gks_scale", C.c_double), ("gks_iso_scale", C.c_double), ("suprep_dose", C.c_double),
                ("reserved", C.c_double * 2)]


class Instance(C.Structure):
    _fields_ = [("ncells", C.c_int32), ("n_stim", C.c_int32), ("model", C.c_int32), ("record", C.c_int32),
                ("dx", C.c_double), ("bcl", C.c_double), ("s1_start", C.c_double), ("s1_duration", C.c_double),
                ("s1_strength", C.c_double), ("s1_beats", C.c_int32), ("reserved0", C.c_int32),
                ("t_stop", C.c_double), ("ecg_x0", C.c_double), ("act_threshold", C.c_double),
                ("s2_base", C.c_double), ("s2_offset", C.c_double), ("s2_duration", C.c_double),
                ("s2_strength", C.c_double), ("s2_cell0", C.c_int32), ("s2_ncells", C.c_int32),
                ("track_vmax", C.c_int32), ("reserved1", C.c_int32)]


class BatchParams(C.Structure):
    _fields_ = [("dt", C.c_double), ("v0", C.c_double), ("precision", C.c_int32), ("max_beats", C.c_int32),
                ("rec_every", C.c_int64), ("threads", C.c_int32), ("ctas", C.c_int32), ("stream", C.c_void_p)]


class Geometry(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("dx", C.c_double),
                ("cell_type", C.c_void_p), ("fibre", C.c_void_p), ("d_fibre", C.c_double),
                ("d_trans", C.c_double), ("coeff_1d", C.c_void_p)]


class Protocol(C.Structure):
    _fields_ = [("bcl", C.c_double), ("s1_start", C.c_double), ("s1_duration", C.c_double),
                ("s1_strength", C.c_double), ("s1_beats", C.c_int32), ("reserved0", C.c_int32),
                ("s1_mask", C.c_void_p), ("s1_onset", C.c_void_p), ("s2_time", C.c_double),
                ("s2_duration", C.c_double), ("s2_strength", C.c_double), ("s2_mask", C.c_void_p)]


class SimParams(C.Structure):
    _fields_ = [("dt", C.c_double), ("v0", C.c_double), ("precision", C.c_int32), ("detect", C.c_int32),
                ("model", Model), ("act_threshold", C.c_double), ("vmin_ok", C.c_double), ("vmax_ok", C.c_double),
                ("stream", C.c_void_p)]


_lib = None


class SurConfig(C.Structure):
    _fields_ = [("dvdt_max", C.c_double), ("kappa", C.c_double), ("vstep_max", C.c_double), ("use_net", C.c_int32),
                ("nsub", C.c_int32), ("foot_dvdt", C.c_double), ("foot_v", C.c_double)]


def lib():
    """Load liblqt.so (building it first if this checkout has no build yet)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        from . import build as _build
        _build.build()
    L = C.CDLL(LIB_PATH)
    P, I, I32, I64, D = C.c_void_p, C.c_int, C.c_int32, C.c_int64, C.c_double
    sig = {
        "lqt_last_error": ([], C.c_char_p),
        "lqt_model_preset": ([I, C.POINTER(Model)], I),
        "lqt_initial_state": ([D, P], I),
        "lqt_cells_create": ([I64, P, I, C.POINTER(Model), D, P, C.POINTER(P)], I),
        "lqt_cells_destroy": ([P], None),
        "lqt_cells_count": ([P], I64),
        "lqt_cells_set_state": ([P, P], I),
        "lqt_cells_get_state": ([P, P], I),
        "lqt_cells_set_inputs": ([P, P, P], I),
        "lqt_cells_update": ([P, I64], I),
        "lqt_cells_get_v": ([P, P], I),
        "lqt_cells_get_dvdt": ([P, P], I),
        "lqt_cells_get_currents": ([P, P], I),
        "lqt_cells_output_states": ([P, I64, I64, P], I),
        "lqt_cells_readin_states": ([P, I64, I64, P], I),
        "lqt_state_write_text": ([P, I64, P], I),
        "lqt_state_read_text": ([P, I64, P], I),
        "lqt_batch_create": ([C.POINTER(BatchParams), I32, P, P, P, I32, P, C.POINTER(P)], I),
        "lqt_batch_destroy": ([P], None),
        "lqt_batch_num_cells": ([P], I64),
        "lqt_batch_run": ([P], I),
        "lqt_batch_get_detect": ([P, P, P, P, P, P], I),
        "lqt_batch_get_record": ([P, I32, P, P, P, I64, C.POINTER(I64)], I),
        "lqt_batch_get_record_currents": ([P, I32, P, P, I64, C.POINTER(I64)], I),
        "lqt_batch_get_vmax": ([P, P], I),
        "lqt_batch_get_state": ([P, P], I),
        "lqt_batch_set_state": ([P, P], I),
        "lqt_batch_last_run_ms": ([P], D),
        "lqt_batch_num_bad": ([P], I64),
    }
    optional = {
        "lqt_sim_create": ([C.POINTER(SimParams), C.POINTER(Geometry), C.POINTER(P)], I),
        "lqt_sim_destroy": ([P], None),
        "lqt_sim_set_protocol": ([P, C.POINTER(Protocol)], I),
        "lqt_sim_num_tissue": ([P], I64),
        "lqt_sim_tissue_index": ([P, P], I),
        "lqt_sim_step": ([P, I64], I),
        "lqt_sim_step_async": ([P, I64], I),
        "lqt_sim_sync": ([P], I),
        "lqt_sim_time": ([P], D),
        "lqt_sim_get_v": ([P, P, I], I),
        "lqt_sim_get_state": ([P, P], I),
        "lqt_sim_set_state": ([P, P], I),
        "lqt_sim_set_electrodes": ([P, I32, P, I32], I),
        "lqt_sim_get_ecg": ([P, I64, P, P, C.POINTER(I64)], I),
        "lqt_sim_get_detect": ([P, P, P, P], I),
        "lqt_sim_check": ([P, C.POINTER(I64)], I),
        "lqt_sim_checkpoint": ([P, C.c_char_p], I),
        "lqt_sim_restore": ([P, C.c_char_p], I),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes, f.restype = args, res
    for name, (args, res) in optional.items():
        if hasattr(L, name):
            f = getattr(L, name)
            f.argtypes, f.restype = args, res
    _lib = L
    return L


class CFile:
    """A C stdio stream (FILE*) for the entry points that take one, opened
    and closed through the C library the native code uses."""

    _libc = None

    def __init__(self, path: str, mode: str):
        if CFile._libc is None:
            libc = C.CDLL(None)
            libc.fopen.argtypes = [C.c_char_p, C.c_char_p]
            libc.fopen.restype = C.c_void_p
            libc.fclose.argtypes = [C.c_void_p]
            CFile._libc = libc
        self.ptr = CFile._libc.fopen(os.fsencode(path), mode.encode())
        if not self.ptr:
            raise OSError(f"cannot open {path} ({mode})")

    def close(self):
        if self.ptr:
            CFile._libc.fclose(self.ptr)
            self.ptr = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def check(code: int, where: str):
    if code != OK:
        msg = lib().lqt_last_error()
        raise LqtError(code, where, msg.decode() if msg else "")


def model(preset: str | dict = "default", **over) -> Model:
    m = Model()
    if isinstance(preset, str):
        check(lib().lqt_model_preset(PRESET[preset], C.byref(m)), "lqt_model_preset")
    else:
        for k, v in preset.items():
            setattr(m, k, float(v))
    for k, v in over.items():
        setattr(m, k, float(v))
    return m
