"""Host-side logic of the batched autotuner (no GPU): the batch signature it
caches results under and the seeded sample it times."""
import numpy as np

from qrdm_gb300.autotune import DEFAULT_CANDIDATES, _sample, signature


def test_signature_rounds_shapes_to_powers_of_two():
    a = [(100, 50), (200, 90), (700, 300), (2000, 512)]
    b = [(110, 48), (190, 100), (690, 280), (1900, 500)]  # same octaves
    assert signature(a) == signature(b)
    assert signature(a) != signature(a + [(64, 64)])  # the count is part of it
    assert signature(a)[0] == 4


def test_sample_keeps_the_largest_problems_and_is_seeded():
    rng = np.random.default_rng(0)
    shapes = [(int(m), int(n)) for m, n in zip(rng.integers(32, 2048, 1000), rng.integers(32, 512, 1000))]
    s1 = _sample(shapes, 100, seed=3)
    s2 = _sample(shapes, 100, seed=3)
    assert s1 == s2 and len(s1) == 100 and len(set(s1)) == 100
    flops = np.array([2.0 * m * n * n for m, n in shapes])
    top = set(np.argsort(-flops)[:25].tolist())
    assert top <= set(s1)  # a quarter of the sample: the largest problems
    assert _sample(shapes[:50], 100) == list(range(50))  # small batches: all problems


def test_default_candidates_are_valid_launches():
    for nb, prec in DEFAULT_CANDIDATES:
        assert prec in ("fp64", "mixed")
        assert 1 <= nb <= 64 and (prec == "fp64" or nb <= 32)
