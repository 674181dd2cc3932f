"""The tensor-train core sweep order (Auxiliar.py:413-527 cpd_cores), on CPU:
which inner core is decomposed at each step, which factor is fixed, and which
step's result is kept for its core."""
import pytest

tt = pytest.importorskip("tensorfox_gb300.tt")


@pytest.mark.parametrize("L,epochs,want", [
    (3, 1, []),
    (3, 2, [(1, 2, True), (1, 0, True)]),            # epochs made odd: 2 -> 3
    (3, 3, [(1, 2, True), (1, 0, True)]),
    (4, 1, [(2, 0, True)]),
    (4, 3, [(2, 0, False), (1, 2, True), (2, 0, True)]),
    (5, 1, [(2, 0, True), (3, 0, True)]),
    (5, 3, [(2, 0, False), (3, 0, False), (2, 2, True), (1, 2, True), (2, 0, True), (3, 0, True)]),
    (6, 5, [(2, 0, False), (3, 0, False), (4, 0, False), (3, 2, False), (2, 2, False), (1, 2, False),
            (2, 0, False), (3, 0, False), (4, 0, False), (3, 2, True), (2, 2, True), (1, 2, True),
            (2, 0, True), (3, 0, True), (4, 0, True)]),
])
def test_sweep_schedule(L, epochs, want):
    assert tt.sweep_schedule(L, epochs) == want
