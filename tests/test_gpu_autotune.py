"""Launch shapes of the fused MD kernel: every (threads per CTA, lanes per atom) shape the
autotuner may pick gives the oracle's forces (relative RMS 1e-5), the tuner leaves the state
as it found it and caches its choice per workload."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("block_threads,lanes", [(512, 1), (640, 4), (896, 2), (1024, 4), (1024, 8), (256, 16)])
def test_every_launch_shape_matches_oracle(block_threads, lanes):
    from kups_gb300 import md
    from test_gpu_core import md_state, oracle_forces, small_batch

    W = small_batch()
    prop = md.make_velocity_verlet_step(steps_per_call=5, block_threads=block_threads, min_lanes_per_atom=lanes)
    out = prop(None, md_state(W))
    pos = out.particles.positions.cpu().numpy()
    _, f, _ = oracle_forces(W, pos)
    gf = out.particles.forces.cpu().numpy()
    assert np.sqrt(np.mean((gf - f) ** 2) / np.mean(f**2)) < 1e-5


def test_autotuner_restores_state_and_caches(tmp_path):
    from kups_gb300 import autotune, md
    from test_gpu_core import md_state, small_batch

    W = small_batch()
    prop = md.make_baoab_langevin_step()
    packed = md.pack(md_state(W))
    before = [t.clone() for t in (packed.pos4, packed.mom4, packed.frc4)]
    cache = str(tmp_path / "tuned.json")
    shape = autotune.autotune_md(prop, packed, steps=10, cache_file=cache, block_threads=(512, 1024),
                                 min_lanes=(1, 2))
    for a, b in zip(before, (packed.pos4, packed.mom4, packed.frc4)):
        assert torch.equal(a, b)
    assert (shape.block_threads, shape.min_lanes_per_atom) in {(512, 1), (512, 2), (1024, 1), (1024, 2)}
    assert (prop.block_threads, prop.min_lanes_per_atom) == (shape.block_threads, shape.min_lanes_per_atom)
    assert len(shape.table) == 4 and all(ms is not None for _, _, ms in shape.table)
    autotune._CACHE.clear()
    other = md.make_baoab_langevin_step()
    again = autotune.autotune_md(other, packed, cache_file=cache)  # served from the file
    assert (again.block_threads, again.min_lanes_per_atom) == (shape.block_threads, shape.min_lanes_per_atom)
