"""TEST INFRASTRUCTURE — NOT PART OF THE PRODUCT.

numpy FP64 restatement of the velocity-Verlet step of moving point charges
that ElectroMag/src/Particle_System.cpp:109-190 describes (emgVerletStep,
with emgFieldsAdd :72-102 and BoundToBox :28-66).  The reference's template
is never instantiated and cannot be (magneto_k carries a trailing
semicolon, include/Magnetics.h:25; Vector3 has no arithmetic operators), so
there is no reference output to pin this against: parity for this step is
unpinned and rests on this restatement and on closed-form cases.

Every particle reads the other particles' start-of-step states, as the
reference's loop reads dynCharges[j] (which it never updates).  Only tests/
import this module.
"""
import numpy as np

ELECTRO_K = 8.987551787e9   # include/Electrostatics.h:27
MAGNETO_K = 1e-7            # include/Magnetics.h:25


def verlet_step(dyn, accel, charges, box_min, box_max, dt):
    """dyn (n, 8) {x, y, z, q, vx, vy, vz, m}, accel (n, 3), charges (p, 4):
    returns the new (dyn, accel) in float64."""
    d = np.asarray(dyn, np.float64)
    a = np.asarray(accel, np.float64)
    ch = np.asarray(charges, np.float64).reshape(-1, 4)
    n = len(d)
    dt2 = dt / 2
    v = d[:, 4:7] + a * dt2
    r = d[:, :3] + v * dt
    # static charges
    rs = r[:, None, :] - ch[None, :, :3]
    l2 = (rs ** 2).sum(-1)
    E = (ch[None, :, 3, None] * rs / (l2 * np.sqrt(l2))[..., None]).sum(1)
    # other particles at their start-of-step positions and velocities
    rd = r[:, None, :] - d[None, :, :3]
    l2 = (rd ** 2).sum(-1)
    np.fill_diagonal(l2, np.inf)
    inv3 = 1.0 / (l2 * np.sqrt(l2))
    w = d[None, :, 3] * inv3                      # q_j / |r|^3
    E += (w[..., None] * rd).sum(1)
    B = (w[..., None] * np.cross(d[None, :, 4:7], rd)).sum(1)
    E *= ELECTRO_K
    B *= MAGNETO_K
    q, m = d[:, 3:4], d[:, 7:8]
    acc = (q * E + q * np.cross(v, B)) / m
    v = v + acc * dt2
    lo = np.asarray(box_min, np.float64)
    hi = np.asarray(box_max, np.float64)
    for c in range(3):                 # upper walls first, as BoundToBox
        over = r[:, c] > hi[c]
        r[over, c] = 2 * hi[c] - r[over, c]
        v[over, c] = -v[over, c]
    for c in range(3):
        under = r[:, c] < lo[c]
        r[under, c] = 2 * lo[c] - r[under, c]
        v[under, c] = -v[under, c]
    out = d.copy()
    out[:, :3] = r
    out[:, 4:7] = v
    return out, acc
