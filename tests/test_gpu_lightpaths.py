"""Light paths (sst_trace_light_paths) against the oracle's restatement of
LightPathCache.TraceAllPaths: the same emitter / background selection, emitted rays, random walk
with importance transport and the same vertex records, per path on the same seeds.  Paths whose
FP32 decisions flip (a grazing hit, a Russian-roulette draw on the edge) may differ; the rest
agree to FP32 tolerance."""
import numpy as np
import pytest

from oracle import pyoracle as O
from seesharp_gb300 import workloads

pytestmark = pytest.mark.gpu


def _compare(sc, n, max_depth, seed=4711, it=3):
    sc.Prepare()
    gf, gi, gl, st = sc.native.trace_light_paths(seed, it, n, max_depth)
    o = O.OracleScene.from_scene(sc)
    of, oi, ol = o.light_paths(seed, it, max_depth, n)
    # the oracle's record: floats (position 3, normal 3, shading normal 3, pdfFrom, pdfRev, weight 3,
    # maxRoughness, fromBackground), ints (mesh, prim, depth, pathId)
    same_len = gl == ol
    assert same_len.mean() >= 0.99, same_len.mean()
    good = 0
    for p in np.nonzero(same_len)[0]:
        L = gl[p]
        g, r = gf[p, :L], of[p, :L]
        ok = np.allclose(g[:, 0:9], r[:, 0:9], rtol=1e-3, atol=1e-3)
        ok &= np.allclose(g[:, 9:11], r[:, 9:11], rtol=2e-3, atol=1e-6)
        ok &= np.allclose(g[:, 12:15], r[:, 11:14], rtol=2e-3, atol=1e-5)
        ok &= np.allclose(g[:, 15], r[:, 14], rtol=1e-5, atol=1e-6)
        ok &= np.array_equal(gi[p, :L, 4], r[:, 15].astype(np.int32))
        ok &= np.array_equal(gi[p, :L, 0:4], oi[p, :L, 0:4])
        good += bool(ok)
    assert good >= 0.98 * same_len.sum(), (good, same_len.sum())
    assert np.all(gf[:, :, 11] == 0)   # no next-event pdf callback
    return gl, st


def test_light_paths_cornell_box():
    gl, st = _compare(workloads.cornell_box(32, 32), 4000, 6)
    assert np.bincount(gl).size >= 5 and st.numRays > 0


def test_light_paths_sphere_field_with_background():
    """GenericMaterials (metallic, transmissive) and the environment map as a light."""
    sc = workloads.sphere_field(12, 32, 32, level=3)
    gl, _ = _compare(sc, 6000, 8)


@pytest.mark.parametrize("name", ["GlossyLight", "DirectIllumTransmit"])
def test_light_paths_validation_scenes(name):
    sc, _, _ = workloads.VALIDATION_SCENES[name](32, 32)
    _compare(sc, 3000, 5)
