"""Recipe for oracle/_ref/libpicurv_ref.so: the reference's own particle-path C code, compiled
unmodified from its sources, for pinning the CPU restatement (picurv_oracle.c).  Test
infrastructure, run only where the reference's sources are present.

Compiled translation units (the reference's src/ and include/ as they are):
  walkingsearch.c   the walking search (every function of the walk)
  ParticleSwarm.c   UpdateParticleWeights and the swarm field registration
  interpolation.c   center->corner, trilinear interpolation, scatter of P to the grid
  ParticleMotion.c  position update, status reset, LocateAllParticlesInGrid_TEST, removals,
                    particle counts
  grid.c            the rank's bounding box (ComputeLocalBoundingBox)
  setup.c           BinarySearchInt64 (the PID lookup of LocateAllParticlesInGrid_TEST)
plus tests/petsc_stub/minipetsc.c (a one-rank stand-in for PETSc's containers and MPI) and
oracle/ref_harness.c (entry points that build a one-rank UserCtx and call the reference's
functions).  Flags: -O2 -ffp-contract=off (no fused multiply-adds; the reference's objects are
built without FMA) and -fvisibility=hidden with --gc-sections, so only the harness's ref_*
entry points are exported and functions of these files that the path never reaches (grid-file
reading, migration between ranks, VTK output) drop out with their PETSc dependencies.

Usage: python oracle/ref_build.py [--reference DIR]   (default: /root/reference)
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
STUB = os.path.join(ROOT, "tests", "petsc_stub")
OUT_DIR = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT_DIR, "libpicurv_ref.so")
DEFAULT_REFERENCE = "/root/reference"
UNITS = ["walkingsearch.c", "ParticleSwarm.c", "interpolation.c", "ParticleMotion.c", "grid.c", "setup.c"]
CFLAGS = ["-std=gnu11", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-fvisibility=hidden",
          "-ffunction-sections", "-fdata-sections", "-w"]


def reference_dir(explicit: str | None = None) -> str | None:
    d = explicit or os.environ.get("PICURV_REFERENCE", DEFAULT_REFERENCE)
    return d if os.path.isfile(os.path.join(d, "src", "walkingsearch.c")) else None


def sources(ref: str) -> list[str]:
    return [os.path.join(ref, "src", u) for u in UNITS] + [os.path.join(STUB, "minipetsc.c"),
                                                         os.path.join(HERE, "ref_harness.c")]


def up_to_date(ref: str) -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    deps = sources(ref) + [os.path.join(STUB, "minipetsc.h"), __file__]
    return all(os.path.getmtime(p) <= t for p in deps)


def build(reference: str | None = None, force: bool = False) -> str | None:
    """Builds oracle/_ref/libpicurv_ref.so; returns its path, or None without the reference."""
    ref = reference_dir(reference)
    if ref is None:
        return None
    if not force and up_to_date(ref):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    objs = []
    for src in sources(ref):
        obj = os.path.join(OUT_DIR, os.path.basename(src)[:-2] + ".o")
        cmd = ["gcc", *CFLAGS, "-I", STUB, "-I", os.path.join(ref, "include"), "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compiling {src} failed:\n{r.stderr}")
        objs.append(obj)
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = ["gcc", "-shared", "-Wl,--gc-sections", "-Wl,-z,defs", "-o", tmp, *objs, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"linking {LIB} failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    for o in objs:
        os.remove(o)
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=None)
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args()
    out = build(a.reference, a.force)
    print(out if out else "reference sources not found: oracle/_ref not built")
    sys.exit(0)
