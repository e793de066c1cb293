"""The learned count kernel's search identities, checked on the CPU.

The count kernel (csrc/learned.cu, learned_count_kernel) walks an Eytzinger
(breadth-first) tree over the interior knots kn[1..B-1] with `knot <= key`
deciding right, and then reads the segment's end knots off the leaf index:
the last right turn is `leaf >> ffs(leaf)` (slot 0 holds kn[0] when there is
none) and the last left turn `leaf >> ffs(~leaf)` (0: kn[B]).  This restates
the tree layout of learned_prepare_kernel and those two formulas in Python and
checks them against a brute-force search, with duplicate knots and keys below,
on and above the knots."""
import random

import pytest


def _ffs(x: int) -> int:
    x &= 0xFFFFFFFF
    return (x & -x).bit_length() if x else 0


def _eytzinger(kn, B):
    d = B.bit_length() - 1
    tree = [kn[0]] + [None] * (B - 1)  # slot 0: the lowest knot, as in the kernel's shared memory
    for i in range(1, B):
        level = i.bit_length() - 1
        rank = ((2 * (i - (1 << level)) + 1) << (d - 1 - level)) - 1  # in-order position
        tree[i] = kn[rank + 1]
    return tree, d


@pytest.mark.parametrize("B", [2, 4, 64, 1024, 16384])
def test_leaf_names_the_segment_and_its_end_knots(B):
    rng = random.Random(B)
    for trial in range(20 if B < 16384 else 3):
        small = trial % 2 == 0  # few distinct values: many equal knots
        kn = sorted(rng.randrange(0, 40) if small else rng.randrange(0, 1 << 63) for _ in range(B + 1))
        tree, d = _eytzinger(kn, B)
        for _ in range(200):
            key = rng.choice([rng.randrange(0, 48), rng.randrange(0, 1 << 64), rng.choice(kn), kn[0] - 1, kn[-1] + 1])
            key = max(0, min(key, (1 << 64) - 1))
            node = 1
            for _level in range(d):
                node = 2 * node + (1 if tree[node] <= key else 0)
            seg = node - B
            assert seg == sum(1 for i in range(1, B) if kn[i] <= key)
            rn, ln = node >> _ffs(node), node >> _ffs(~node)
            assert tree[rn] == kn[seg]
            assert (tree[ln] if ln else kn[B]) == kn[seg + 1]
