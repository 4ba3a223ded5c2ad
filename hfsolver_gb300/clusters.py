"""Seeded synthetic molecules for the benchmarks and tests.

* water(): one H2O, O at the origin, H1 on +x, H2 in the xy-plane, with
  r(OH) = 0.9572 A and angle(HOH) = 104.52 deg.
* water_cluster(n, box, seed): n rigid copies of that water, each with a
  uniformly random orientation (unit quaternion from four normal deviates),
  oxygen centres uniform in a cube of side `box` (A) by rejection sampling with
  every O-O distance >= 2.7 A.  Default box: 8 A scaled by (n/8)^(1/3), i.e.
  the density of 8 waters in an 8 A cube.  Optional Gaussian atom jitter
  (sigma in A).  Draw order: centres, orientations, jitter, from
  numpy.random.default_rng(seed).
* water_batch(count, seed): `count` clusters of U{1..12} waters with
  sigma = 0.05 A jitter, one sub-seed per geometry.
Coordinates are returned in bohr with hfsolver's ang2bohr = 1/0.529177249
(src/constants.f90:43-44).
"""
import numpy as np

ANG2BOHR = 1 / 0.529177249
R_OH = 0.9572
ANGLE_HOH = 104.52


def _water_frame():
    th = np.deg2rad(ANGLE_HOH)
    return np.array([[0.0, 0.0, 0.0], [R_OH, 0.0, 0.0], [R_OH * np.cos(th), R_OH * np.sin(th), 0.0]])


def water():
    """(atno, xyz[bohr]) of the single water molecule."""
    return np.array([8, 1, 1], dtype=np.int32), _water_frame() * ANG2BOHR


def _rotation(q):
    w, x, y, z = q / np.linalg.norm(q)
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def water_cluster(n, box=None, seed=0, jitter=0.0, min_oo=2.7):
    rng = np.random.default_rng(seed)
    if box is None:
        box = 8.0 * (n / 8.0) ** (1.0 / 3.0)
    centres = []
    tries = 0
    while len(centres) < n:
        c = rng.uniform(0.0, box, 3)
        tries += 1
        if tries > 1_000_000:
            raise RuntimeError("could not place the waters; enlarge the box")
        if all(np.linalg.norm(c - o) >= min_oo for o in centres):
            centres.append(c)
    frame = _water_frame()
    xyz = []
    for c in centres:
        R = _rotation(rng.normal(size=4))
        xyz.extend(c + frame @ R.T)
    xyz = np.array(xyz)
    if jitter > 0:
        xyz = xyz + rng.normal(0.0, jitter, xyz.shape)
    atno = np.tile(np.array([8, 1, 1], dtype=np.int32), n)
    return atno, xyz * ANG2BOHR


def water_batch(count=256, seed=0, nmin=1, nmax=12, jitter=0.05):
    rng = np.random.default_rng(seed)
    sizes = rng.integers(nmin, nmax + 1, size=count)
    return [water_cluster(int(s), seed=seed * 100003 + 7919 * (i + 1), jitter=jitter)
            for i, s in enumerate(sizes)]
