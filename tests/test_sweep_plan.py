"""Host logic of the subspace sweep: the anchor plan and the spread pick."""
from hamiltonian_diagonalization_gb300.sweep import pick_spread, subspace_plan


def test_plan_and_spread():
    assert subspace_plan(64) == [0, 1, 2, 3, 4, 6, 12, 24, 39, 51, 63]
    p = subspace_plan(16)
    assert p[0] == 0 and p[-1] == 15 and p == sorted(set(p))
    assert pick_spread([2, 3, 5, 8, 9, 11, 12], 3) == [2, 8, 12]
    assert pick_spread([4, 7], 8) == [4, 7]
