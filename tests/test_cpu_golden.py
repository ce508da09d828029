"""The oracle against the committed golden fixtures (tests/golden/, made by
tests/golden/make_golden.py): every vector is regenerated and compared bit
for bit, so any change to the oracle's arithmetic shows here."""
import os

import numpy as np
import pytest

from tests.golden import make_golden

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def regenerated():
    return make_golden.generate()


def _load(name):
    with np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


def _bits(a):
    a = np.ascontiguousarray(a)
    if a.dtype.fields:
        return a.view(np.uint8)
    return a.view(np.uint32) if a.dtype.itemsize == 4 else a


@pytest.mark.parametrize("name", ["philox", "detmath", "hits_cornell", "hits_instanced", "bvh_cornell",
                                  "film_cornell_bxdf", "film_cornell_nee", "film_cornell_mis",
                                  "film_cornell_mis_all", "film_zoo_mis", "film_volume",
                                  "particles_cornell", "particles_zoo", "particles_instanced", "reference_scenes"])
def test_oracle_reproduces_golden(regenerated, name):
    want = _load(name)
    got = regenerated[name]
    assert set(want) == set(got)
    for k in want:
        assert want[k].shape == np.asarray(got[k]).shape, k
        assert np.array_equal(_bits(want[k]), _bits(np.asarray(got[k], dtype=want[k].dtype))), f"{name}.{k}"


def test_golden_films_are_not_trivial():
    for name in ["film_cornell_bxdf", "film_cornell_nee", "film_cornell_mis", "film_zoo_mis", "film_volume",
                 "particles_cornell", "particles_zoo", "particles_instanced"]:
        f = _load(name)["film"].view(np.float32)
        assert np.count_nonzero(f) > f.size // 4, name
    for name in ["particles_cornell", "particles_zoo", "particles_instanced"]:
        z = _load(name)
        assert z["n"].sum() > 50 and (z["pix"] >= 0).sum() == np.minimum(z["n"], 12).sum(), name
