"""GPU: the k-slab decomposition (fdf_gb300/slabs.py) with real GPU contexts: two rank processes
share the one GPU of the test machine, each with its own context and the whole grid, and exchange
particles and boundary face sums on the host (gloo); no kernel of one rank waits on the other.
fdf_ExtractParticles, fdf_AddParticles and fdf_DepositKFaceLayer carry the ranks' union to the
one-rank oracle's results bit for bit (swarm, removal counts, ParticleCount, P average, face
volume and momentum deposits)."""
import pytest

from tests.test_slabs import run_slabs

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["sinusoidal", "bent_pipe"])
def test_gpu_slab_ranks_equal_one_rank(require_gpu, tmp_path, name):
    run_slabs(tmp_path, name, 2, gpu=True)
