"""GPU, full size: the 128x128x2048 curved pipe with 128M particles and the volume and momentum
face deposits (the largest configuration), against the FP64 oracle on all host cores.

* Plain FP64 form: initial setup and 2 steps of the whole workload, every particle and every
  grid field bit for bit (swarm fields by PID, removal counts, ParticleCount, P average, face
  volume and momentum deposits).
* FP32 form: 200 steps of the whole workload; the oracle steps the particles with PID < 1M (an
  i.i.d. sample; particles do not interact) from the same initial state; per-field errors.
The 96x96x1536 configurations (64M and 16M particles) run the same checks in bench.py's default
line (plain_vs_oracle_full, fp32_errors_cfg3)."""
import os

import pytest

import bench

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(require_gpu):
    from fdf_gb300.context import PicContext
    with PicContext(0) as c:
        yield c


def test_plain_form_full_size_curved_pipe(ctx):
    r = bench.plain_parity_full(ctx, bench.workload("curved_pipe"), 2, os.cpu_count() or 1)
    print(f"[plain FP64 vs oracle, {r['initial_particles']} particles, 2 steps] identical {r['identical']}, "
          f"seconds {r['seconds']}")
    assert r["identical"], {k: v for k, v in r.items() if k != "seconds"}


def test_fp32_form_errors_curved_pipe(ctx):
    r = bench.fp32_errors_full(ctx, bench.workload("curved_pipe"), 200, 1_000_000, os.cpu_count() or 1)
    print(f"[FP32 form vs FP64 oracle, curved pipe, 200 steps] velocity {r['velocity_rel']}, faces "
          f"{r['face_volume_abs_per_particle_volume']}, momentum {r['face_momentum_abs_per_particle_momentum']}, "
          f"other cell {r['particles_in_another_cell']}, one-sided removals {r['particles_removed_by_one_side_only']}")
    assert r["sample_run_equals_full_run"]
    assert r["same_cell_fraction"] >= 0.9999
    assert r["velocity_rel"]["max"] <= 1e-5
    assert r["face_volume_abs_per_particle_volume"]["max"] <= 1e-5
    assert r["face_momentum_abs_per_particle_momentum"]["max"] <= 1e-5
