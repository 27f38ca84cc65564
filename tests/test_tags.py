"""Refinement tags, host part: the 2:1 smoothing (ffv_tags_smooth, criterionsmth.c) against
the reference's own smoothing of the same target levels, for every tag pass the model-5
fixtures hold (generated by tests/golden/make_golden.py from the reference's
interface_location / criterionsplt / criterionsmth)."""
import ctypes

import numpy as np
import pytest

from conftest import golden_names, load_golden
from helpers import mesh_from_golden

from forestfv_public_gb300 import _lib


def level_max(t):
    """LEVEL as inputset.c:106 and m5_input.c:53 form it from the criterion levels."""
    return int(max(t[1], t[3], t[6], t[9], t[12], t[15]))


@pytest.mark.parametrize("name", golden_names(model=5))
def test_smoothing_matches_reference(name, built_lib):
    g = load_golden(name)
    m = mesh_from_golden(g)
    L = _lib.lib()
    assert g["tags"].shape[0] >= 3
    for params, ref in zip(g["tag_params"], g["tags"]):
        split = np.ascontiguousarray(ref[:, 2].astype(np.int32))
        rc = L.ffv_tags_smooth(m.handle, level_max(params), split.ctypes.data)
        assert rc == 0
        assert np.array_equal(split, ref[:, 3]), (name, params)


def test_smoothing_is_two_to_one():
    """After smoothing no face neighbour's target exceeds a leaf's by more than one."""
    from forestfv_public_gb300.mesh import Mesh, uniform_leaves
    m = Mesh((2, 2, 2), uniform_leaves((2, 2, 2), 4))
    rng = np.random.default_rng(3)
    split = rng.integers(1, 7, m.n).astype(np.int32)
    assert _lib.lib().ffv_tags_smooth(m.handle, 6, split.ctypes.data) == 0
    ex = m.export()
    nb, bc = ex["nb"], ex["bc"]
    for c in range(m.n):
        for f in range(6):
            if bc[c, f] == 0:
                for q in nb[c, f]:
                    if q >= 0:
                        assert split[q] - split[c] <= 1
