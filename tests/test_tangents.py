"""Tangents (er_compute_tangents) against the reference's own MikkTSpace
output (tests/golden/reference_tangents.npz, from tests/golden/gen_tangents.py).

Signs must agree everywhere.  Directions agree (cos > 0.9999) on at least
97 % of corners; the rest are at texture-space singular points (the poles
of a sphere mapping, where every face around the vertex has another
tangent direction): the reference keeps each face's own tangent there, this
implementation the angle-weighted mean.
"""
import os

import numpy as np
import pytest

from eleven import _lib

GOLD = os.path.join(os.path.dirname(__file__), "golden", "reference_tangents.npz")


@pytest.mark.parametrize("name", ["uvsphere", "icosphere"])
def test_tangents_match_reference_mikktspace(name):
    G = np.load(GOLD)
    t, s = _lib.compute_tangents(G[f"{name}_P"], G[f"{name}_N"], G[f"{name}_U"])
    assert np.array_equal(s, G[f"{name}_S"])
    cos = (t * G[f"{name}_T"]).sum(-1)
    assert (cos > 0.9999).mean() >= 0.97
    assert np.allclose(np.linalg.norm(t, axis=-1), 1.0, atol=1e-5)
