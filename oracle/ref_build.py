"""Build oracle/_ref/libref_physics.so from the reference's own physics headers.

Recipe: g++ on oracle/ref_physics.cpp with -I <reference checkout> and the
ristra stand-ins in oracle/ref_shim; no reference build system is used.  Only
possible where the reference checkout exists and the environment variable
FLECSALE_REFERENCE names it; elsewhere build_if_available() does nothing.
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT_DIR, "libref_physics.so")


def reference_root() -> str:
    """The reference checkout named by FLECSALE_REFERENCE ("" when unset)."""
    return os.environ.get("FLECSALE_REFERENCE", "")


def available() -> bool:
    r = reference_root()
    return bool(r) and os.path.exists(os.path.join(r, "flecsale", "eqns", "euler_eqns.h"))


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    src = os.path.join(HERE, "ref_physics.cpp")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-fPIC", "-shared",
               "-ffp-contract=off", "-DNDEBUG", "-I", os.path.join(HERE, "ref_shim"), "-I",
               reference_root(), src, "-o", LIB + ".tmp"]
        subprocess.run(cmd, check=True)
        os.replace(LIB + ".tmp", LIB)
    return LIB


def build_if_available() -> str | None:
    if available():
        return build()
    return None
