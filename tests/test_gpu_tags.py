"""Refinement tags on the GPU (ffv_tags: interface_location + criterionsplt on the device,
criterionsmth on the host) against the reference's own tag passes on the same states:
interface layers, raw target levels and smoothed target levels must be identical."""
import numpy as np
import pytest

from conftest import golden_names, load_golden, m5_params
from helpers import mesh_from_golden

from forestfv_public_gb300 import FFVError, Mesh, Solver
from forestfv_public_gb300.mesh import uniform_leaves

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", golden_names(model=5))
def test_tags_match_reference(name, built_lib):
    g = load_golden(name)
    m = mesh_from_golden(g)
    q = m5_params(g)
    s = Solver(model=5, order=int(g["order"]), rk_steps=int(g["rk_steps"]), gamma=q["gamma"],
               pinf=q["pinf"], mu=q["mu"], amin=q["amin"], avf_lim=q["avf_lim"],
               prelax=q["prelax"])
    s.set_mesh(m)
    s.upload_state(np.ascontiguousarray(g["S_final"].T))
    for params, ref in zip(g["tag_params"], g["tags"]):
        split, raw, si = s.tags(params, with_raw=True)
        if params[11]:
            assert np.array_equal(si[0], ref[:, 0]) and np.array_equal(si[1], ref[:, 1]), params
        assert np.array_equal(raw, ref[:, 2]), (params, np.flatnonzero(raw != ref[:, 2])[:10])
        assert np.array_equal(split, ref[:, 3]), params
    s.close()


def test_tags_model0(built_lib):
    """Model 0: uniform level, the relative-jump criterion on cell states (an extension of
    the reference, which has no model-0 branch), no interface layers."""
    m = Mesh((2, 2, 2), uniform_leaves((2, 2, 2), 3))
    s = Solver()
    s.set_mesh(m)
    S = np.zeros((5, m.n))
    S[0], S[4] = 1.0, 2.5
    s.upload_state(S)
    split = s.tags((1, 4, 0, 0, 0.0, 0, 0, 0.0, 0, 0, 0.0, 0, 0, 0, 0, 0, 0))
    assert (split == 4).all()  # one level per smoothing pass at most
    grad = (1, 3, 1, 5, 0.1, 1, 5, 0.1, 0, 0, 0.0, 0, 0, 0, 0, 0, 0)
    assert (s.tags(grad) == 3).all()  # no jumps in a uniform state
    x = m.centroids()
    S[0] = np.where(x[:, 0] < 0.5, 1.0, 0.125)
    s.upload_state(S)
    split, raw, _ = s.tags(grad, with_raw=True)
    jump = np.abs(x[:, 0] - 0.5) < 0.5 / (1 << 2)  # the two cell layers at the discontinuity
    assert (raw[jump] == 5).all() and (raw[~jump] == 3).all()
    assert split.max() == 4  # one level per pass above the mesh
    with pytest.raises(FFVError):
        s.tags((1, 4, 0, 0, 0.0, 0, 0, 0.0, 0, 0, 0.0, 1, 5, 2, 0, 0, 0))
    s.close()
