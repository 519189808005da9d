"""The multiply-high division the GPU kernels use to find element coordinates
(ElemIndexer in csrc/sdg_stage_warp.cuh) and face-flux tasks (FaceTasks in
csrc/sdg_stage.cuh): q = floor(e * m / 2^32) with m = floor((2^32 - 1) / d) + 1
equals floor(e / d) whenever d > 1 and e * d < 2^32 -- the condition under
which the kernels use it.  Checked here in exact integer arithmetic at the
edges of that range and on seeded random samples."""
import numpy as np


def umulhi_div(e: int, d: int) -> int:
    m = (0xFFFFFFFF // d + 1) & 0xFFFFFFFF
    return (e * m) >> 32


def test_multiply_high_matches_division_in_its_range():
    rng = np.random.default_rng(20261203)
    divisors = list(range(2, 300)) + [2 ** k for k in range(1, 16)] + \
        [int(x) for x in rng.integers(2, 1 << 16, 300)]
    for d in divisors:
        top = ((1 << 32) - 1) // d  # the largest e with e * d < 2^32
        es = {0, 1, d - 1, d, d + 1, top, top - 1, top - d, max(0, top - 1 - d)}
        es |= {int(x) for x in rng.integers(0, top + 1, 64)}
        for e in es:
            assert umulhi_div(e, d) == e // d, (e, d)


def test_the_kernels_fall_back_outside_it():
    """d = 1 has no 32-bit constant (the kernels divide then), and past
    e * d = 2^32 the quotient can be one too large: with d = 3 (r = m d - 2^32
    = 2) it is at e = 2^31, where e / d + e r / (d 2^32) reaches the next
    integer."""
    assert (0xFFFFFFFF // 1 + 1) & 0xFFFFFFFF == 0
    e, d = 1 << 31, 3
    assert e % d == d - 1 and e * d >= 1 << 32
    assert umulhi_div(e, d) == e // d + 1
