"""The drop-in integrator plugin's material translation (spica_gb300/plugins/
material_probe.h), run on the compiled reference's own BSDFs: it must read back the
record of every material the GPU renders, with the reference's smooth-limit rule for
rough dielectrics (bsdfs/roughdielectric.cc:58), and refuse what the GPU cannot
render instead of approximating it.  Needs the reference tree (CPU only)."""
import os

import numpy as np
import pytest

from oracle import spo
from spica_gb300 import scenes

CASES = {
    "lambert": scenes.lambert(0.3, 0.5, 0.7),
    "conductor": scenes.conductor_f0(0.2, (0.9, 0.6, 0.3)),
    "conductor_beckmann": [scenes.MAT_CONDUCTOR_BECKMANN] + scenes.conductor_f0(0.15, (0.5, 0.7, 0.95))[1:],
    "dielectric": scenes.dielectric(1.5),
    "beckmann": scenes.rough_dielectric(0.25, 1.5, "beckmann"),
    "ggx": scenes.rough_dielectric(0.15, 1.33, "ggx"),
    "beckmann_sharp": scenes.rough_dielectric(0.02, 2.4, "beckmann"),
    "ggx_rough": scenes.rough_dielectric(0.9, 1.1, "ggx"),
    "plastic": scenes.plastic((0.6, 0.3, 0.2), (0.4, 0.4, 0.4), 1.5),
    "plastic_tinted": scenes.plastic((0.1, 0.8, 0.5), (0.05, 0.02, 0.03), 1.3),
    "plastic_high_index": scenes.plastic((0.2, 0.2, 0.2), (0.9, 0.1, 0.3), 5.5),
    "plastic_no_specular": scenes.plastic((0.1, 0.8, 0.5), (0.0, 0.0, 0.0), 1.7),
    "plastic_no_diffuse": scenes.plastic((0.0, 0.0, 0.0), (0.5, 0.5, 0.5), 2.0),
}


@pytest.fixture(scope="module")
def ref():
    if not os.path.isdir(spo.REF_TREE):
        pytest.skip("reference tree not present on this host")
    spo.build("ref")
    return spo.Oracle("ref")


@pytest.mark.parametrize("name", sorted(CASES))
def test_probe_reads_back_the_material(ref, name):
    m = np.asarray(CASES[name], np.float64)
    rec, why = ref.probe_material(m)
    assert why is None, why
    np.testing.assert_allclose(rec, m.astype(np.float32), rtol=2e-6, atol=1e-7)


def test_zero_roughness_is_the_smooth_dielectric(ref):
    rec, why = ref.probe_material(scenes.rough_dielectric(0.0, 1.5, "ggx"))
    assert why is None
    np.testing.assert_array_equal(rec, np.float32(scenes.dielectric(1.5)))


def test_plastic_without_a_positive_lobe_is_refused(ref):
    # Kd only, index 4: the reference's diffuse term (1 - Fdr) turns negative there
    rec, why = ref.probe_material(scenes.plastic((0.1, 0.8, 0.5), (0.0, 0.0, 0.0), 4.0))
    assert rec is None and "plastic" in why
