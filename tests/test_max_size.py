"""Lists addressed beyond 2^32 entries.  The lists are slot-major with the capacity as the stride,
and the density-active workload's two cell shells give every full list 255 slots (its particles
hold ~125 entries), so a simulation of capacity 40,000,000 addresses slot k of particle i at
k x 40,000,000 + i, past 2^32 for k >= 108.  The density-active 1M workload stepped in such a simulation must give the bits of
the same workload in a simulation of capacity 1M (offsets below 2^31) and of the cell-walking
path (PBD_FLAG_FULL_WALK: no stored list), frame by frame."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CAP = 40_000_000


def test_lists_beyond_2_to_32_entries(need_gpu, pbd, scenes):
    params, pos, vel, _ = scenes.workload("fluid_1m_dense", pbd)
    params.flags |= pbd.FLAG_TRACK_IDS
    n = len(pos)
    walk = pbd.Params.from_buffer_copy(params)
    walk.flags |= pbd.FLAG_FULL_WALK
    runs = []
    for prm, cap in ((params, CAP), (params, n), (walk, n)):
        with pbd.Sim(prm, cap) as sim:
            sim.add_particles(pos, vel)
            out = []
            for f in range(2):
                sim.step(1)
                sim.sync()
                st = sim.state()
                out.append((st["x"], st["v"], st["ids"]))
                if cap == CAP and f == 0:   # the longest lists reach slots whose offsets pass 2^32
                    _, cnt, _ = sim.neighbours(0)
                    assert (int(cnt.max()) - 1) * CAP > 2 ** 32, int(cnt.max())
            runs.append(out)
    for other in runs[1:]:
        for (xa, va, ia), (xb, vb, ib) in zip(runs[0], other):
            assert np.array_equal(ia, ib)
            assert np.array_equal(xa, xb) and np.array_equal(va, vb)
