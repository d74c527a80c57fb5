"""The FP64 gradient oracle against central finite differences of its own
double-precision image (same Philox words, i.e. common random numbers).

Albedo and emission enter a path's radiance polynomially, so central
differences match the analytic gradient to rounding.  Roughness moves scatter
directions; with a small step no path changes its hit sequence or lobe, and
the pathwise part of the roughness gradient (the forward-mode tangents of the
miss direction) must match the difference quotient closely.  The lobe-choice
part is a score-function term whose mean is the derivative of the lobe
probabilities: a small step with common random numbers flips no coin, so it
is checked against the CUDA adjoint and, at many samples, against central
differences of the GPU render instead."""
import copy

import numpy as np
import pytest

import oracle
from raydar_gb300 import scenegen
from tests.helpers import shrink

W = H = 20
SPP = 4
BOUNCES = 6
SEED = 77


@pytest.fixture(scope="module")
def setup():
    scene = shrink(scenegen.c4_diff().scene, W, H)
    rng = np.random.default_rng(5)
    dl = rng.uniform(-1.0, 1.0, (H, W, 3)).astype(np.float32)
    ga, gr, ge, img, gp = oracle.gradient(scene.to_c(), 0, SPP, BOUNCES, SEED, dl, threads=8, pathwise=True)
    return scene, dl, ga, gr, ge, img, gp


def _loss(scene, dl):
    _, _, _, img = oracle.gradient(scene.to_c(), 0, SPP, BOUNCES, SEED, dl, threads=8)
    return float((img * dl.astype(np.float64)).sum())


def _fd(scene, dl, set_param, base, eps):
    lo, hi = copy.deepcopy(scene), copy.deepcopy(scene)
    a = np.float32(base - eps)
    b = np.float32(base + eps)
    set_param(lo, a)
    set_param(hi, b)
    return (_loss(hi, dl) - _loss(lo, dl)) / (float(b) - float(a))


def test_image_matches_the_float_oracle(setup):
    scene, dl, ga, gr, ge, img, gp = setup
    acc, _ = oracle.render(scene.to_c(), 0, SPP, BOUNCES, SEED, threads=8)
    ref = acc[..., :3].astype(np.float64) / SPP
    # the double path follows the float path except on rare borderline decisions
    close = np.abs(img - ref) <= 1e-4 * (1 + np.abs(ref))
    assert close.mean() > 0.99


def test_albedo_and_emission_gradients_match_central_differences(setup):
    scene, dl, ga, gr, ge, img, gp = setup
    checked = 0
    for j in (0, 3, 11):  # the ground and two spheres
        for c in range(3):
            base = float(scene.objects[j].material.albedo[c])

            def set_alb(s, v, j=j, c=c):
                s.objects[j].material.albedo = s.objects[j].material.albedo.copy()
                s.objects[j].material.albedo[c] = v

            fd = _fd(scene, dl, set_alb, base, 1e-3)
            assert abs(fd - ga[j, c]) <= 1e-5 * (1 + abs(ga[j, c])), (j, c, fd, ga[j, c])
            checked += 1
    j = len(scene.objects) - 1  # an emissive sphere: E = colour * strength, colour 1
    base = float(scene.objects[j].material.emission_strength)

    def set_em(s, v):
        s.objects[j].material.emission_strength = float(v)

    fd = _fd(scene, dl, set_em, base, 1e-2)
    assert abs(fd - ge[j].sum()) <= 1e-5 * (1 + abs(ge[j].sum()))
    assert checked == 9 and np.abs(ga).sum() > 0 and np.abs(ge).sum() > 0


def test_metal_roughness_gradient_matches_central_differences(setup):
    scene, dl, ga, gr, ge, img, gp = setup
    metals = [i for i, o in enumerate(scene.objects)
              if o.material.metallic == 1.0 and o.material.roughness > 0.1 and abs(gp[i]) > 0]
    assert metals, "the scene has a rough metal that the image sees"
    j = max(metals, key=lambda i: abs(gp[i]))
    base = float(scene.objects[j].material.roughness)

    def set_r(s, v):
        s.objects[j].material.roughness = float(v)

    fd = _fd(scene, dl, set_r, base, 1e-5)
    assert abs(fd - gp[j]) <= 2e-2 * abs(gp[j]), (j, fd, gp[j])


def test_lobe_choice_terms_are_separate_from_the_pathwise_part(setup):
    """Objects of the Specular class (roughness 0.5, not metal, not glass)
    take the roughness coin on every hit, so their gradient has a lobe term;
    metals take no roughness coin, so theirs differs from the pathwise part
    only through the Fresnel coins of glass hits further along the path."""
    scene, dl, ga, gr, ge, img, gp = setup
    spec = [i for i, o in enumerate(scene.objects) if o.material.metallic == 0.0 and
            o.material.transmission == 0.0 and o.material.roughness == 0.5]
    assert spec and any(abs(gr[i] - gp[i]) > 1e-9 * (1 + abs(gr[i])) for i in spec)
    # objects with roughness 0 (glass) have no roughness gradient of either kind: d(r^2)/dr = 0 there
    glass = [i for i, o in enumerate(scene.objects) if o.material.roughness == 0.0]
    assert glass and all(gr[i] == 0.0 and gp[i] == 0.0 for i in glass)


def test_the_float_evaluation_agrees_with_double_on_a_well_conditioned_scene(setup):
    """oracle.gradient(fp32=True) takes the same derivative with each path's
    intermediates in float (the precision of the CUDA adjoint).  On the c4
    scene, where no path's derivative is ill-conditioned and the double
    replay loses no hit, the two evaluations agree to float rounding
    (measured 4e-5 relative on the roughness gradient, 6 bounces)."""
    scene, dl, ga, gr, ge, img, _ = setup
    fa, fr, fe, fimg = oracle.gradient(scene.to_c(), 0, SPP, BOUNCES, SEED, dl, threads=8, fp32=True)
    assert oracle.gradient.lost_paths == 0
    for f, d in ((fa, ga), (fr, gr), (fe, ge), (fimg, img)):
        assert np.linalg.norm(f - d) <= 1e-4 * np.linalg.norm(d) + 1e-9
