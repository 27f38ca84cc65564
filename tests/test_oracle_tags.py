"""The numpy restatement of the reference's refinement tags (oracle/tags.py) against the
reference's own tag passes on the model-5 fixtures' final states: interface layers, raw
target levels and smoothed target levels identical."""
import numpy as np
import pytest

from conftest import golden_names, load_golden, m5_params
from helpers import geometry_from_golden

from forestfv_public_gb300 import leaves_from_paths
from oracle import tags as T


@pytest.mark.parametrize("name", golden_names(model=5))
def test_tag_restatement_matches_reference(name):
    g = load_golden(name)
    geo = geometry_from_golden(g)
    lv = leaves_from_paths(tuple(g["ntrees"]), g["root"], g["level"],
                           g["adrs"][:, 2:].astype(np.int64))
    S = np.ascontiguousarray(g["S_final"].T)
    m5 = m5_params(g)
    for params, ref in zip(g["tag_params"], g["tags"]):
        SI, raw, split = T.tags(S, geo, m5, tuple(params), lv.level, lv.tree_ijk, lv.cell_ijk)
        if params[11]:
            assert np.array_equal(SI[0], ref[:, 0]) and np.array_equal(SI[1], ref[:, 1]), params
        assert np.array_equal(raw, ref[:, 2]), (params, np.flatnonzero(raw != ref[:, 2])[:10])
        assert np.array_equal(split, ref[:, 3]), params
