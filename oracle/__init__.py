"""ORACLE — test infrastructure only (see hydro_oracle.cpp).

Loads liboracle_hydro.so, the CPU restatement of the reference hydro tasks.
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it,
always as the checker or the timed CPU baseline, never as the product path.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB = os.path.join(HERE, "liboracle_hydro.so")
SRC = os.path.join(HERE, "hydro_oracle.cpp")
_L = None


def build(force: bool = False) -> str:
    """g++ -O2 without floating-point contraction, OpenMP over cells/faces."""
    hdr = os.path.join(ROOT, "include", "flecsale_gb300.h")
    stale = (not os.path.exists(LIB) or os.path.getmtime(LIB) < max(
        os.path.getmtime(SRC), os.path.getmtime(hdr), os.path.getmtime(__file__)))
    if force or stale:
        cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-fPIC", "-shared",
               "-fopenmp", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
               SRC, "-o", LIB + ".tmp"]
        subprocess.run(cmd, check=True)
        os.replace(LIB + ".tmp", LIB)
    return LIB


def load() -> C.CDLL:
    global _L
    if _L is None:
        from flecsale_gb300.hydro import (FluxView, GradientView, MeshView, Params,
                                          StateView)
        L = C.CDLL(build())
        vp, dp, mp, sp = C.c_void_p, C.POINTER(C.c_double), C.POINTER(MeshView), C.POINTER(StateView)
        gp, fp, pp = C.POINTER(GradientView), C.POINTER(FluxView), C.POINTER(Params)
        i64p = C.POINTER(C.c_int64)
        L.oracle_evaluate_time_step.argtypes = [mp, sp, pp, C.c_double, dp]
        L.oracle_evaluate_time_step.restype = C.c_int
        L.oracle_evaluate_gradients.argtypes = [mp, sp, gp, pp]
        L.oracle_evaluate_gradients.restype = None
        L.oracle_evaluate_fluxes.argtypes = [mp, sp, gp, fp, pp]
        L.oracle_evaluate_fluxes.restype = None
        L.oracle_apply_update.argtypes = [mp, pp, C.c_double, C.c_double, fp, sp, dp, i64p]
        L.oracle_apply_update.restype = C.c_int
        L.oracle_set_threads.argtypes = [C.c_int32]
        L.oracle_set_threads.restype = None
        L.oracle_max_threads.argtypes = []
        L.oracle_max_threads.restype = C.c_int32
        L.oracle_run.argtypes = [mp, pp, sp, C.c_int64, C.c_int, dp, i64p, i64p]
        L.oracle_run.restype = C.c_int
        L.oracle_state_from_pressure.argtypes = [C.c_int32, C.c_double, C.c_double, dp, dp,
                                                 dp, dp, dp]
        L.oracle_state_from_pressure.restype = None
        L.oracle_face_flux.argtypes = [C.c_int32, C.c_int32, dp, dp, dp, dp]
        L.oracle_face_flux.restype = None
        L.oracle_update_cell.argtypes = [C.c_int32, C.c_double, C.c_double, dp, dp]
        L.oracle_update_cell.restype = None
        _L = L
    return _L
