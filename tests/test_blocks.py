"""Block-partitioned contraction (the Dagger decomposition of
ext/MuscleDaggerExt/binary_einsum.jl:64-119), host side: the block plan's
validation, its tasks, the decomposition itself summed block by block on the
CPU with the oracle against the whole contraction, and the sharding of output
blocks over two gloo ranks whose outputs add up to the whole result."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from muscle_gb300 import ArgumentError, DimensionMismatch
from muscle_gb300.blocks import BlockPlan
from oracle import muscle_ref as ref

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# (ia, shape_a, ib, shape_b, ic, block sizes)
CASES = [
    # matrix product, every label split
    (["i", "k"], (8, 12), ["k", "j"], (12, 6), ["i", "j"], {"i": 4, "k": 3, "j": 2}),
    # two contracted labels, output permuted, one label unsplit
    (["i", "j", "k", "l"], (4, 6, 4, 2), ["k", "m", "l", "n"], (4, 3, 2, 5), ["n", "i", "m", "j"],
     {"k": 2, "l": 1, "i": 2, "n": 5}),
    # hyperindex: b kept in the output and split
    (["i", "b", "k"], (6, 4, 8), ["k", "b", "j"], (8, 4, 3), ["i", "j", "b"], {"b": 1, "k": 4}),
    # vector times matrix, the contracted label split into four blocks
    (["k"], (12,), ["k", "j"], (12, 6), ["j"], {"k": 3, "j": 3}),
    # outer product: nothing contracted, one pair per output block
    (["i"], (6,), ["j"], (4,), ["j", "i"], {"i": 2, "j": 2}),
]


def _arrays(case, seed=0, cx=True):
    ia, sa, ib, sb, ic, bs = case
    rng = np.random.default_rng(seed)
    mk = lambda s: np.asfortranarray(rng.standard_normal(s) + (1j * rng.standard_normal(s) if cx else 0))
    return mk(sa), mk(sb)


def _blocked_on_cpu(plan, a, b, tasks):
    """Sums every task's block pairs with the oracle into a zero output."""
    ic = [i.tag for i in plan.ic]
    c = np.zeros([plan.ext[i] for i in plan.ic], dtype=np.result_type(a, b), order="F")
    ia, ib = [i.tag for i in plan.ia], [i.tag for i in plan.ib]
    for t in tasks:
        view = c[plan._slices(plan.ic, dict(zip(plan.ic, t.out_block)))]
        for sa, sb in t.pairs:
            view += ref.contract(a[sa], ia, b[sb], ib, ic)
    return c


@pytest.mark.parametrize("case", CASES)
def test_decomposition_sums_to_the_whole(case):
    ia, sa, ib, sb, ic, bs = case
    a, b = _arrays(case)
    plan = BlockPlan(ia, sa, ib, sb, ic, bs)
    tasks = plan.tasks()
    n_out = np.prod([plan.nblocks[i] for i in plan.ic])
    n_sum = np.prod([plan.nblocks[i] for i in plan.sum_labels]) if plan.sum_labels else 1
    assert len(tasks) == n_out and all(len(t.pairs) == n_sum for t in tasks)
    got = _blocked_on_cpu(plan, a, b, tasks)
    want = ref.contract(a, ia, b, ib, ic)
    assert ref.rel_fro(got, want) <= 1e-14


@pytest.mark.parametrize("world", [2, 3, 5])
def test_assignment_covers_every_block_once(world):
    ia, sa, ib, sb, ic, bs = CASES[0]
    plan = BlockPlan(ia, sa, ib, sb, ic, bs)
    every = [t.out_block for t in plan.tasks()]
    got = [[t.out_block for t in plan.assign(r, world)] for r in range(world)]
    flat = [x for g in got for x in g]
    assert sorted(flat) == sorted(every) and len(flat) == len(set(flat))
    sizes = [len(g) for g in got]
    assert max(sizes) - min(sizes) <= 1  # equal-work blocks: dealt evenly


def test_validation():
    with pytest.raises(ArgumentError):
        BlockPlan(["i", "k"], (8, 12), ["k", "j"], (12, 6), ["i", "j"], {"k": 5})  # 5 does not divide 12
    with pytest.raises(ArgumentError):
        BlockPlan(["i", "k"], (8, 12), ["k", "j"], (12, 6), ["i", "j"], {"z": 2})  # no such label
    with pytest.raises(ArgumentError):
        BlockPlan(["i", "k"], (8, 12), ["k", "j"], (12, 6), ["i", "x"], {})  # x in neither operand
    with pytest.raises(DimensionMismatch):
        BlockPlan(["i", "k"], (8, 12), ["k", "j"], (10, 6), ["i", "j"], {})
    with pytest.raises(ArgumentError):
        BlockPlan(["i", "k"], (8, 12), ["k", "j"], (12, 6), ["i", "j"], {}).assign(2, 2)


CHILD = r"""
import json, os, sys
sys.path.insert(0, {root!r})
sys.path.insert(0, os.path.join({root!r}, "muscle.jl_gb300", "python"))
import numpy as np
import torch, torch.distributed as dist
from tests import test_blocks as tb
from muscle_gb300.blocks import BlockPlan
from oracle import muscle_ref as ref
dist.init_process_group("gloo")
rank, ws = dist.get_rank(), dist.get_world_size()
case = tb.CASES[0]
ia, sa, ib, sb, ic, bs = case
a, b = tb._arrays(case, seed=3)
plan = BlockPlan(ia, sa, ib, sb, ic, bs)
mine = plan.assign(rank, ws)
part = tb._blocked_on_cpu(plan, a, b, mine)
t = torch.from_numpy(np.ascontiguousarray(part))
dist.all_reduce(t)                     # replicas own disjoint output blocks
whole = ref.contract(a, ia, b, ib, ic)
err = ref.rel_fro(t.numpy(), np.ascontiguousarray(whole))
dist.destroy_process_group()
print(json.dumps({{"rank": rank, "blocks": len(mine), "err": err}}))
"""


def test_output_blocks_sharded_over_two_gloo_ranks(tmp_path):
    script = tmp_path / "child.py"
    script.write_text(CHILD.format(root=ROOT))
    env = dict(os.environ, MASTER_ADDR="127.0.0.1", MASTER_PORT="29583", WORLD_SIZE="2", CUDA_VISIBLE_DEVICES="")
    procs = [subprocess.Popen([sys.executable, str(script)], env=dict(env, RANK=str(r)), stdout=subprocess.PIPE,
                              stderr=subprocess.PIPE, text=True) for r in range(2)]
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=240)
        assert p.returncode == 0, err[-2000:]
        outs.append(json.loads(out.strip().splitlines()[-1]))
    assert sorted(o["rank"] for o in outs) == [0, 1]
    assert sum(o["blocks"] for o in outs) == 2 * 3 and all(o["blocks"] == 3 for o in outs)
    assert all(o["err"] <= 1e-14 for o in outs)
