"""Test infrastructure: the CPU oracle for the depth-fusion path.

* ``oracle/kifi_oracle.c`` -- the C restatement of the reference algorithm,
  and ``oracle/kifi_oracle_k64.c``, its fusion path with 64-bit voxel keys
  (both built into ``oracle/_build/libkifi_oracle.so``), wrapped by
  ``oracle.cpu``.
* ``oracle/_ref`` -- the reference's own CPU code compiled by
  ``oracle/build_ref.py``, wrapped by ``oracle.ref``.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs import
this package; the shipped library never does.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
ORACLE_LIB = os.path.join(BUILD, "libkifi_oracle.so")


def build_oracle():
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(HERE, f) for f in ("kifi_oracle.c", "kifi_oracle_k64.c")]
    cmd = ["gcc", "-std=c11", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
           "-Wall", "-Wno-unused-function", "-o", ORACLE_LIB] + srcs + ["-lm"]
    subprocess.check_call(cmd)
    return ORACLE_LIB


def build(with_reference=True):
    """Build the C restatement and, when its sources are available, the
    reference CPU library.  Returns (oracle_lib, reference_lib_or_None)."""
    lib = build_oracle()
    ref = None
    if with_reference:
        from . import build_ref
        ref = build_ref.build()
    return lib, ref
