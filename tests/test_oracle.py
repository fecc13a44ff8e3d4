"""CPU tests of the oracle: known answers derived from the reference's code, sort stability,
cell-range invariants and FP32-vs-FP64 agreement.  No GPU."""
import numpy as np
import pytest

from helpers import by_id, maxdiff, workload


def test_expand_bits_kat(oracle_mod):
    # Hash.h:10-16 spreads 10 bits over 30: 0x3FF -> 0x09249249
    assert oracle_mod.expand_bits(0x3FF) == 0x09249249
    assert oracle_mod.expand_bits(0) == 0
    assert oracle_mod.expand_bits(1) == 1
    assert oracle_mod.expand_bits(2) == 0b1000
    assert oracle_mod.expand_bits(3) == 0b1001


def test_morton_kat(oracle_mod):
    # Hash.h:21-29: x<<2 | y<<1 | z, clamped to [0, 1023], truncated
    assert oracle_mod.morton(1.0, 0.0, 0.0) == 4
    assert oracle_mod.morton(0.0, 1.0, 0.0) == 2
    assert oracle_mod.morton(0.0, 0.0, 1.0) == 1
    assert oracle_mod.morton(1.99, 0.5, 0.2) == 4
    assert oracle_mod.morton(-5.0, -0.1, 0.0) == 0
    assert oracle_mod.morton(5000.0, 0.0, 0.0) == oracle_mod.expand_bits(1023) << 2
    assert oracle_mod.morton(127.9, 127.9, 127.9) == (1 << 21) - 1


def _front(oracle_mod, pbd, scenes, shape, seed, box=16, precision="f32"):
    p, pos, vel = workload(pbd, scenes, shape=shape, box=box, seed=seed, flags_extra=pbd.FLAG_TRACK_IDS)
    o = oracle_mod.Oracle(p, pos.shape[0], precision)
    o.add_particles(pos, vel)
    o.step_phase(oracle_mod.PHASE_FRONT)
    return o, p, pos, vel


def test_sort_is_stable_sort_of_keys(oracle_mod, pbd, scenes):
    o, p, pos, vel = _front(oracle_mod, pbd, scenes, (9, 7, 5), seed=3)
    d = o.debug()
    st = o.state()
    # predicted positions before the sort: recompute the keys of p* in the input order
    keys_in = d["keys"][np.argsort(d["perm"])]
    ref_perm = np.argsort(keys_in, kind="stable")
    assert np.array_equal(d["perm"], ref_perm)
    assert np.all(np.diff(d["keys"].astype(np.int64)) >= 0)
    assert np.array_equal(st["ids"], d["perm"])


def test_cell_ranges_partition(oracle_mod, pbd, scenes):
    o, p, pos, vel = _front(oracle_mod, pbd, scenes, (10, 10, 10), seed=4)
    G = 1 << 18
    d = o.debug(ncells=G)
    keys, cs, ce = d["keys"], d["cell_start"], d["cell_end"]
    n = len(keys)
    occupied = np.unique(keys)
    for c in occupied:
        idx = np.nonzero(keys == c)[0]
        assert cs[c] == idx[0]
        if not (c == n - 1 and n >= 2):   # SortReorder.h:183-184 overwrites this one end
            assert ce[c] == idx[-1] + 1
    empty = np.setdiff1d(np.arange(G), occupied)
    assert np.all(cs[empty] == 0xFFFFFFFF)




def test_f32_matches_f64_one_step(oracle_mod, pbd, scenes):
    p, pos, vel = workload(pbd, scenes, shape=(8, 8, 8), seed=5, flags_extra=pbd.FLAG_TRACK_IDS)
    a = oracle_mod.Oracle(p, pos.shape[0], "f32")
    b = oracle_mod.Oracle(p, pos.shape[0], "f64")
    for o in (a, b):
        o.add_particles(pos, vel)
        o.step(1)
    sa, sb = by_id(a.state()), by_id(b.state())
    assert maxdiff(sa["x"][:, :3], sb["x"][:, :3]) < 1e-4
    assert maxdiff(sa["v"][:, :3], sb["v"][:, :3]) < 1e-2


def test_lists_match_bruteforce(oracle_mod, pbd, scenes):
    """The list of findContacts is every particle of the 27 cells around p*, self excluded."""
    p, pos, vel = workload(pbd, scenes, shape=(6, 6, 6), seed=6)
    o = oracle_mod.Oracle(p, pos.shape[0], "f32")
    o.add_particles(pos, vel)
    o.step_phase(oracle_mod.PHASE_LISTS)
    lst, cnt, con = o.neighbours(64)
    st = o.state()
    pp = st["p"][:, :3]
    cell = np.floor(pp).astype(np.int64)
    for i in range(0, len(pp), 7):
        near = np.all(np.abs(cell - cell[i]) <= 1, axis=1)
        near[i] = False
        assert set(lst[i, :cnt[i]].tolist()) == set(np.nonzero(near)[0].tolist())
        assert cnt[i] == con[i]
