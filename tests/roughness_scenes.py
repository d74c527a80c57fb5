"""Scenes on which the roughness gradient is well defined for central
differences: no ray of the weighted pixels can cross a silhouette or a
total-internal-reflection edge under a small roughness step, so the image is
smooth in the roughness (pathwise part) and in the probabilities of the coins
that pick a lobe (score-function part).

  lone_metal     a rough metal sphere (roughness 0.3) in the sky: camera ->
                 sphere -> the perturbed reflection -> sky.  Only the pathwise
                 part.
  lone_specular  a sphere of the Specular class (roughness 0.5, not metal):
                 the roughness coin picks diffuse with P = r^2, else the
                 perturbed reflection.  Pathwise + roughness-coin parts.
  glass_floor    a rough metal sphere above a huge glass cube (ior 1.5),
                 3 bounces: camera -> sphere -> floor, where Schlick's R (a
                 function of the perturbed direction) decides reflection to
                 the sky or refraction into the cube (radiance 0 within the
                 bounce limit).  Pathwise + Fresnel-coin parts.

`pixel_weights` returns dL/dimage: nonzero only on the pixels whose primary
ray hits the sphere away from its rim (and, for glass_floor, whose mirror
direction reaches the floor obliquely, well away from the cone that reflects
back into the sphere), so no weighted path nears a discontinuity.  For
lone_specular the weight is +-1 by the sign of (E[diffuse] - E[specular]) of
the pixel's sky radiance (estimated from the mean diffuse direction, 2/3 of
the normal, against the mirror direction), so the lobe-probability
derivative of every pixel adds up instead of cancelling."""
import numpy as np

from raydar_gb300.scene import Camera, Material, Object, Scene, World

SKY = World("SkyColor", np.array([0.53, 0.8, 0.92], np.float32), np.array([1.0, 1.0, 1.0], np.float32))
ALBEDO = np.array([0.9, 0.8, 0.7], np.float32)


def lone_metal(size=96):
    cam = Camera.new([0.0, 0.5, -4.0], [0.0, 0.0, 0.0], [0.0, 1.0, 0.0], size, size, 0.01, 1000.0, fov=40.0)
    m = Material(albedo=ALBEDO.copy(), roughness=0.3, metallic=1.0)
    return Scene(cam, SKY, [Object("Sphere", np.zeros(3, np.float32), 1.0, m)]), 0, 4


def lone_specular(size=96):
    cam = Camera.new([0.0, 0.5, -4.0], [0.0, 0.0, 0.0], [0.0, 1.0, 0.0], size, size, 0.01, 1000.0, fov=40.0)
    m = Material(albedo=ALBEDO.copy(), roughness=0.5)
    return Scene(cam, SKY, [Object("Sphere", np.zeros(3, np.float32), 1.0, m)]), 0, 4


def glass_floor(size=96):
    cam = Camera.new([0.0, 1.8, -2.2], [0.0, 1.0, 0.0], [0.0, 1.0, 0.0], size, size, 0.01, 1000.0, fov=16.0)
    metal = Material(albedo=ALBEDO.copy(), roughness=0.3, metallic=1.0)
    glass = Material(albedo=np.array([0.95, 0.95, 0.95], np.float32), roughness=0.0, transmission=1.0, ior=1.5)
    objs = [Object("Sphere", np.array([0.0, 1.0, 0.0], np.float32), 0.5, metal),
            Object("Cube", np.array([0.0, -500.0, 0.0], np.float32), 1000.0, glass)]
    return Scene(cam, SKY, objs), 0, 3


def _primary_dirs(scene):
    cam = scene.camera
    W, H = cam.resolution_x, cam.resolution_y
    ip = cam.inverse_proj_matrix.reshape(4, 4).T.astype(np.float64)
    iv = cam.inverse_view_matrix.reshape(4, 4).T.astype(np.float64)
    ys, xs = np.mgrid[0:H, 0:W]
    u, v = xs / W, 1.0 - ys / H
    clip = np.stack([2 * u - 1, 2 * v - 1, -np.ones_like(u), -np.ones_like(u)], -1)
    c = clip @ ip.T
    c = c / c[..., 3:4]
    w = c @ iv.T
    d = -w[..., :3]
    return d / np.linalg.norm(d, axis=-1, keepdims=True)


def pixel_weights(name, scene):
    """dL/dimage (H x W x 3 float32) for the scene `name` (see the module doc)."""
    o = scene.camera.position.astype(np.float64)
    d = _primary_dirs(scene)
    sph = scene.objects[0]
    c, rad = sph.center.astype(np.float64), float(sph.size)
    oc = o - c
    b = d @ oc
    disc = b * b - (oc @ oc - rad * rad)
    hit = disc > 0
    t = -b - np.sqrt(np.where(hit, disc, 0.0))
    p = o + t[..., None] * d
    n = (p - c) / rad
    cos_in = -(d * n).sum(-1)
    mask = hit & (t > 0) & (cos_in > 0.5)
    if name == "glass_floor":
        u = d - 2 * (d * n).sum(-1, keepdims=True) * n  # mirror direction
        # reaches the floor (y = 0) obliquely: incidence between 55 and 75 degrees, away from grazing
        down = -u[..., 1]
        mask &= (down > np.cos(np.radians(75))) & (down < np.cos(np.radians(55)))
        # the continuation below the floor passes the sphere's mirror image (centre y -> -y) with room
        # for the roughness perturbation (|offset| <= r^2 = 0.09 rad over the distance travelled)
        cm = c * np.array([1.0, -1.0, 1.0])
        w = cm - p
        along = (w * u).sum(-1)
        dist = np.linalg.norm(w - along[..., None] * u, axis=-1)
        mask &= (along < 0) | (dist > rad + 0.12 * np.linalg.norm(w, axis=-1) + 0.05)
    wts = np.zeros(d.shape[:2] + (3,), np.float32)
    wts[mask] = 1.0
    if name == "lone_specular":
        u = d - 2 * (d * n).sum(-1, keepdims=True) * n
        diff = (2.0 / 3.0) * n[..., 1] - u[..., 1]  # E[d_y] of the diffuse lobe minus the mirror's
        sign = np.where(np.abs(diff) > 0.1, -np.sign(diff), 0.0)  # the sky darkens with d_y
        wts *= sign[..., None].astype(np.float32)
    return wts
