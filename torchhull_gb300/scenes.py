"""Seeded synthetic scenes for visual-hull requests.

torchhull's own tests and benchmarks render Armadillo masks through OpenGL
(``data/generate_dataset.py:120-183``), which cannot run here, so the inputs
are made analytically instead: a union of ellipsoids (and thin capsules for
fine structure), seen by pinhole cameras on a sphere looking at the origin.
A mask pixel is 1 when the ray through the pixel centre hits a primitive.

Camera conventions follow the reference's dataset generator and its pixel
conventions (``image_utils.h:62-82``):

* ``"opengl"``: transform = P @ V with P the OpenGL perspective matrix of
  ``generate_dataset.py:13-30`` (near 0.1, far 1000); pixel ``(x, y)`` covers
  NDC ``((x + 0.5) / W * 2 - 1, (y + 0.5) / H * 2 - 1)``, so row 0 is the bottom.
* ``"opencv"``: transform = K @ E with K of ``generate_dataset.py:33-50`` and
  E the OpenGL view conjugated into a +z-forward, y-down camera; pixel
  ``(x, y)`` covers ``(u, v) = (x + 0.5, y + 0.5)``, so row 0 is the top.

Masks are computed in float64 with torch on any device; the same seed gives
the same scene and cameras everywhere.
"""

from __future__ import annotations

import dataclasses
import math

import numpy as np
import torch


@dataclasses.dataclass
class Scene:
    centers: np.ndarray  # [E,3]
    rotations: np.ndarray  # [E,3,3] local -> world
    semi_axes: np.ndarray  # [E,3]
    capsule_a: np.ndarray  # [C,3]
    capsule_b: np.ndarray  # [C,3]
    capsule_r: np.ndarray  # [C]


@dataclasses.dataclass
class Cameras:
    transforms: np.ndarray  # [B,4,4] float64, K @ T
    origins: np.ndarray  # [B,3] camera centres
    cam_to_world: np.ndarray  # [B,3,3] rotation, columns = camera axes in world
    fov: float  # vertical field of view, radians
    height: int
    width: int
    convention: str


def _random_rotation(rng: np.random.Generator) -> np.ndarray:
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array(
        [
            [1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
            [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
            [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)],
        ]
    )


def make_scene(seed: int, n_ellipsoids: int, n_capsules: int = 0) -> Scene:
    rng = np.random.default_rng(seed)
    centers = rng.uniform(-0.5, 0.5, size=(n_ellipsoids, 3))
    semi = rng.uniform(0.15, 0.45, size=(n_ellipsoids, 3))
    rots = np.stack([_random_rotation(rng) for _ in range(n_ellipsoids)]) if n_ellipsoids else np.zeros((0, 3, 3))
    mid = rng.uniform(-0.5, 0.5, size=(n_capsules, 3))
    direction = rng.normal(size=(n_capsules, 3))
    direction /= np.maximum(np.linalg.norm(direction, axis=1, keepdims=True), 1e-12)
    half = rng.uniform(0.1, 0.4, size=(n_capsules, 1))
    radius = rng.uniform(0.01, 0.03, size=n_capsules)
    return Scene(centers, rots, semi, mid - half * direction, mid + half * direction, radius)


def _look_at(eye: np.ndarray) -> np.ndarray:
    """World -> camera rotation for an OpenGL camera (looks down -z, y up) at eye, aimed at the origin."""
    forward = -eye / np.linalg.norm(eye)
    up = np.array([0.0, 1.0, 0.0])
    if abs(float(np.dot(forward, up))) > 0.99:
        up = np.array([0.0, 0.0, 1.0])
    right = np.cross(forward, up)
    right /= np.linalg.norm(right)
    true_up = np.cross(right, forward)
    return np.stack([right, true_up, -forward])  # rows = camera axes


def make_cameras(
    seed: int,
    n: int,
    radius: float,
    fov_deg: float,
    height: int,
    width: int,
    convention: str = "opengl",
) -> Cameras:
    if convention not in ("opengl", "opencv"):
        raise ValueError(f"unknown convention {convention!r}")
    rng = np.random.default_rng(seed + 7919)
    fov = math.radians(fov_deg)
    aspect = width / height
    golden = math.pi * (3.0 - math.sqrt(5.0))
    transforms = np.zeros((n, 4, 4))
    origins = np.zeros((n, 3))
    c2w = np.zeros((n, 3, 3))
    for i in range(n):
        zc = 1.0 - 2.0 * (i + 0.5) / n
        rc = math.sqrt(max(0.0, 1.0 - zc * zc))
        phi = golden * i
        d = np.array([rc * math.cos(phi), zc, rc * math.sin(phi)]) + rng.normal(0.0, 0.05, size=3)
        d /= np.linalg.norm(d)
        eye = radius * d
        rot = _look_at(eye)  # world -> GL camera
        view = np.eye(4)
        view[:3, :3] = rot
        view[:3, 3] = -rot @ eye
        if convention == "opengl":
            near, far = 0.1, 1000.0
            t = math.tan(fov / 2.0)
            proj = np.array(
                [
                    [1.0 / (t * aspect), 0.0, 0.0, 0.0],
                    [0.0, 1.0 / t, 0.0, 0.0],
                    [0.0, 0.0, -(far + near) / (far - near), -(2.0 * far * near) / (far - near)],
                    [0.0, 0.0, -1.0, 0.0],
                ]
            )
            transforms[i] = proj @ view
            c2w[i] = rot.T
        else:
            flip = np.diag([1.0, -1.0, -1.0, 1.0])
            ext = flip @ view
            t = math.tan(fov / 2.0)
            k = np.array(
                [
                    [(width / 2.0) / (t * aspect), 0.0, width / 2.0, 0.0],
                    [0.0, (height / 2.0) / t, height / 2.0, 0.0],
                    [0.0, 0.0, 1.0, 0.0],
                    [0.0, 0.0, 0.0, 1.0],
                ]
            )
            transforms[i] = k @ ext
            c2w[i] = ext[:3, :3].T
        origins[i] = eye
    return Cameras(transforms, origins, c2w, fov, height, width, convention)


def _ray_directions(cams: Cameras, i: int, device: torch.device) -> torch.Tensor:
    h, w = cams.height, cams.width
    t = math.tan(cams.fov / 2.0)
    aspect = w / h
    ys, xs = torch.meshgrid(
        torch.arange(h, dtype=torch.float64, device=device),
        torch.arange(w, dtype=torch.float64, device=device),
        indexing="ij",
    )
    if cams.convention == "opengl":
        dx = ((xs + 0.5) / w * 2.0 - 1.0) * t * aspect
        dy = ((ys + 0.5) / h * 2.0 - 1.0) * t
        dz = -torch.ones_like(dx)
    else:
        f = (h / 2.0) / t
        dx = (xs + 0.5 - w / 2.0) / f
        dy = (ys + 0.5 - h / 2.0) / f
        dz = torch.ones_like(dx)
    d_cam = torch.stack([dx, dy, dz], dim=-1).reshape(-1, 3)
    rot = torch.as_tensor(cams.cam_to_world[i], dtype=torch.float64, device=device)
    d = d_cam @ rot.T
    return d / torch.linalg.norm(d, dim=1, keepdim=True)


def _hits_ellipsoids(o: torch.Tensor, d: torch.Tensor, scene: Scene) -> torch.Tensor:
    dev = d.device
    hit = torch.zeros(d.shape[0], dtype=torch.bool, device=dev)
    for c, r, a in zip(scene.centers, scene.rotations, scene.semi_axes, strict=True):
        rt = torch.as_tensor(r.T, dtype=torch.float64, device=dev)
        inv_a = torch.as_tensor(1.0 / a, dtype=torch.float64, device=dev)
        ol = (rt @ (o - torch.as_tensor(c, dtype=torch.float64, device=dev))) * inv_a
        dl = (d @ rt.T) * inv_a
        qa = (dl * dl).sum(1)
        qb = 2.0 * (dl @ ol)
        qc = float((ol * ol).sum()) - 1.0
        disc = qb * qb - 4.0 * qa * qc
        t_far = (-qb + torch.sqrt(torch.clamp(disc, min=0.0))) / (2.0 * qa)
        hit |= (disc >= 0.0) & (t_far > 0.0)
    return hit


def _hits_capsules(o: torch.Tensor, d: torch.Tensor, scene: Scene) -> torch.Tensor:
    dev = d.device
    hit = torch.zeros(d.shape[0], dtype=torch.bool, device=dev)

    def dist_to_ray(q: torch.Tensor) -> torch.Tensor:  # q: [N,3]
        s = torch.clamp(((q - o) * d).sum(1), min=0.0)
        return torch.linalg.norm(q - (o + s[:, None] * d), dim=1)

    for pa, pb, rad in zip(scene.capsule_a, scene.capsule_b, scene.capsule_r, strict=True):
        p0 = torch.as_tensor(pa, dtype=torch.float64, device=dev)
        v = torch.as_tensor(pb - pa, dtype=torch.float64, device=dev)
        w0 = o - p0
        vv = float(v @ v)
        b = d @ v
        e = float(v @ w0)
        dd = d @ w0
        denom = vv - b * b
        safe = torch.where(denom.abs() > 1e-12, denom, torch.ones_like(denom))
        t_line = torch.clamp((e - b * dd) / safe, 0.0, 1.0)
        t_line = torch.where(denom.abs() > 1e-12, t_line, torch.zeros_like(t_line))
        t_origin = min(max(e / vv, 0.0), 1.0)
        best = dist_to_ray(p0 + t_line[:, None] * v)
        for t in (0.0, 1.0, t_origin):
            best = torch.minimum(best, dist_to_ray((p0 + t * v).expand_as(d)))
        hit |= best <= rad
    return hit


def render_masks(
    scene: Scene,
    cams: Cameras,
    device: str | torch.device = "cpu",
    dtype: torch.dtype = torch.float32,
) -> torch.Tensor:
    """Masks [B,H,W,1] in {0,1}, one ray per pixel centre."""
    device = torch.device(device)
    out = torch.empty((len(cams.transforms), cams.height, cams.width, 1), dtype=dtype, device=device)
    for i in range(len(cams.transforms)):
        d = _ray_directions(cams, i, device)
        o = torch.as_tensor(cams.origins[i], dtype=torch.float64, device=device)
        hit = _hits_ellipsoids(o, d, scene)
        if len(scene.capsule_r):
            hit |= _hits_capsules(o, d, scene)
        out[i] = hit.reshape(cams.height, cams.width, 1).to(dtype)
    return out


@dataclasses.dataclass
class HullRequest:
    masks: torch.Tensor
    transforms: torch.Tensor
    level: int
    cube_corner_bfl: tuple[float, float, float]
    cube_length: float
    masks_partial: bool
    transforms_convention: str
    unique_verts: bool = True

    def kwargs(self) -> dict:
        return dict(
            masks=self.masks,
            transforms=self.transforms,
            level=self.level,
            cube_corner_bfl=self.cube_corner_bfl,
            cube_length=self.cube_length,
            masks_partial=self.masks_partial,
            transforms_convention=self.transforms_convention,
            unique_verts=self.unique_verts,
        )


def make_request(
    seed: int,
    views: int,
    side: int,
    level: int,
    partial: bool,
    convention: str = "opengl",
    n_ellipsoids: int | None = None,
    n_capsules: int | None = None,
    radius: float | None = None,
    fov_deg: float | None = None,
    device: str | torch.device = "cpu",
    mask_dtype: torch.dtype = torch.float32,
) -> HullRequest:
    """One request of the ellipsoid/capsule family.

    Partial requests put the cameras at radius 1.4 with a 50 degree field of
    view, so the object leaves the frame in many views; full requests use
    radius 2.5 and 40 degrees.
    """
    if n_ellipsoids is None:
        n_ellipsoids = 8 if partial else 3
    if n_capsules is None:
        n_capsules = 20 if partial else 0
    if radius is None:
        radius = 1.4 if partial else 2.5
    if fov_deg is None:
        fov_deg = 50.0 if partial else 40.0
    scene = make_scene(seed, n_ellipsoids, n_capsules)
    cams = make_cameras(seed, views, radius, fov_deg, side, side, convention)
    masks = render_masks(scene, cams, device=device, dtype=mask_dtype)
    transforms = torch.as_tensor(cams.transforms, dtype=torch.float32).to(device)
    return HullRequest(masks, transforms, level, (-1.0, -1.0, -1.0), 2.0, partial, convention, True)


def small_request(device: str | torch.device = "cpu", seed: int = 1) -> HullRequest:
    """3 ellipsoids, 8 OpenGL views of 256x256, level 6, full masks."""
    return make_request(seed, 8, 256, 6, False, "opengl", 3, 0, 2.5, 40.0, device)


def blur_request(device: str | torch.device = "cpu", seed: int = 2) -> HullRequest:
    """5 ellipsoids, 24 OpenCV views of 512x512, level 8 (to be blurred with k=9, sigma=2 first)."""
    return make_request(seed, 24, 512, 8, False, "opencv", 5, 0, 2.5, 40.0, device)


def partial_request(device: str | torch.device = "cpu", seed: int = 3) -> HullRequest:
    """8 ellipsoids + 20 capsules, 32 views of 1024x1024 at radius 1.4 (fov 50), level 9, partial masks."""
    return make_request(seed, 32, 1024, 9, True, "opengl", 8, 20, 1.4, 50.0, device)


def batched_requests(count: int = 64, seed: int = 4, device: str | torch.device = "cpu") -> list[HullRequest]:
    """Heterogeneous requests: views U{4..48}, side U{256,512,768,1024}, level U{6..9}, partial ~ Bernoulli(0.3)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        views = int(rng.integers(4, 49))
        side = int(rng.choice([256, 512, 768, 1024]))
        level = int(rng.integers(6, 10))
        partial = bool(rng.random() < 0.3)
        out.append(make_request(seed * 1000 + i, views, side, level, partial, device=device))
    return out
