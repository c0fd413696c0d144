"""CPU checks of the topology sections of Snapshot and of the exclusion pairs derived from them
(the kinds of hoomd/md/nlist.py:55-73)."""

import numpy as np
import pytest

from hoomd_gb300.md.nlist import excluded_pairs
from hoomd_gb300.snapshot import Snapshot


def chain_snapshot():
    s = Snapshot()
    s.particles.N = 6
    s.bonds.N = 5
    s.bonds.group[:] = [[0, 1], [1, 2], [2, 3], [3, 4], [4, 5]]
    s.angles.N = 1
    s.angles.group[:] = [[0, 1, 2]]
    s.dihedrals.N = 1
    s.dihedrals.group[:] = [[2, 3, 4, 5]]
    s.constraints.N = 1
    s.constraints.group[:] = [[0, 5]]
    s.pairs.N = 1
    s.pairs.group[:] = [[1, 4]]
    s.validate()
    return s


def top(s):
    return {k: getattr(s, k) for k in ("bonds", "angles", "dihedrals", "impropers",
                                       "constraints", "pairs")}


@pytest.mark.parametrize("kinds,expect", [
    (("bond",), [[0, 1], [1, 2], [2, 3], [3, 4], [4, 5]]),
    (("angle",), [[0, 2]]),
    (("dihedral",), [[2, 5]]),
    (("constraint",), [[0, 5]]),
    (("special_pair",), [[1, 4]]),
    (("1-3",), [[0, 2], [1, 3], [2, 4], [3, 5]]),
    (("1-4",), [[0, 3], [1, 4], [2, 5]]),
    ((), []),
])
def test_exclusion_kinds(kinds, expect):
    got = excluded_pairs(top(chain_snapshot()), kinds, 6)
    assert got.tolist() == expect


def test_union_is_sorted_and_unique():
    got = excluded_pairs(top(chain_snapshot()), ("bond", "1-3", "angle"), 6)
    rows = [tuple(x) for x in got.tolist()]
    assert rows == sorted(set(rows)) and len(rows) == 9


def test_validate_rejects_bad_groups():
    s = chain_snapshot()
    s.bonds.group[0] = [0, 9]
    with pytest.raises(ValueError, match="tag >= N"):
        s.validate()
