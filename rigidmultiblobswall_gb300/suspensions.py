"""Seeded synthetic suspensions of rigid multiblob shells above a wall.

Geometry follows the reference's structure files: a 12-blob shell is the
icosahedron on a sphere of radius R (multi_bodies/Structures/shell_N_12_Rg_1.vertex)
and a 42-blob shell is the once-subdivided icosahedron (edge midpoints pushed
to the sphere; shell_N_42_Rg_0_8913_Rh_1.vertex, R = 0.8913).  The blob radius
is half the minimum inter-blob distance, the convention of
multi_bodies/examples/Mobility_Prod_Timing/main.py:123-126.  The vertex sets
are generated here from that construction (no reference data is read).

Workloads (numpy.random.default_rng(seed) with seed = workload index):
  blobs_wall_matvec  2048 free blobs, a=0.5, x,y ~ U[0,64a], z ~ U[1.5a,10a]
  shells_42_256      256 shells x 42 blobs (10,752 blobs), x,y ~ U[0,60R], z ~ U[1.2R,5R]
  shells_12_1024     1024 shells x 12 blobs (12,288 blobs), R=1, a=0.4, x,y ~ U[0,120R],
                     z ~ U[1.2R,5R]: the 60R box of the 256-shell workload cannot hold
                     1024 centres 2R+2a apart in that slab, so the side is doubled,
                     which keeps the 256-shell workload's bodies per unit area
  shells_42_4096     4096 shells x 42 blobs (172,032 blobs), area fraction 0.3, z ~ U[1.1R,3R]
  shells_42_batch    64 independent suspensions of 42-blob shells, body counts ~ U{16..512};
                     each placed like shells_42_256 in a box of side 60R sqrt(max(n,256)/256)
"""
import numpy as np

R42 = 0.8912655971483167


def icosahedron(radius=1.0):
    """12 vertices: poles at +-z and two rings of 5 at z = +-radius/sqrt(5)."""
    zr = 1.0 / np.sqrt(5.0)
    rr = 2.0 / np.sqrt(5.0)
    v = [np.array([0.0, 0.0, 1.0])]
    for k in range(5):
        t = np.deg2rad(72.0 * (k + 1))
        v.append(np.array([rr * np.cos(t), rr * np.sin(t), zr]))
    for k in range(5):
        t = np.deg2rad(36.0 + 72.0 * k)
        v.append(np.array([rr * np.cos(t), rr * np.sin(t), -zr]))
    v.append(np.array([0.0, 0.0, -1.0]))
    return radius * np.array(v)


def icosphere_42(radius=R42):
    """Once-subdivided icosahedron: the 12 vertices plus the 30 edge midpoints
    projected on the sphere."""
    base = icosahedron(1.0)
    d = np.linalg.norm(base[:, None, :] - base[None, :, :], axis=-1)
    edge = d[d > 1e-9].min()
    mids = []
    for i in range(12):
        for j in range(i + 1, 12):
            if abs(d[i, j] - edge) < 1e-6:
                m = 0.5 * (base[i] + base[j])
                mids.append(m / np.linalg.norm(m))
    assert len(mids) == 30
    return radius * np.concatenate([base, np.array(mids)])


def blob_radius_of(shell):
    """Half the minimum inter-blob distance."""
    d = np.linalg.norm(shell[:, None, :] - shell[None, :, :], axis=-1)
    return 0.5 * d[d > 0].min()


def random_quaternions(rng, n):
    q = rng.standard_normal((n, 4))
    return q / np.linalg.norm(q, axis=1)[:, None]


def rotation_matrices(q):
    """Rotation matrices of unit quaternions (s, p) as in
    quaternion_integrator/quaternion.py:42-51 (vectorised)."""
    q = np.asarray(q, dtype=np.float64).reshape(-1, 4)
    s, p0, p1, p2 = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    diag = s * s - 0.5
    R = np.empty((q.shape[0], 3, 3))
    R[:, 0, 0] = p0 * p0 + diag
    R[:, 0, 1] = p0 * p1 - s * p2
    R[:, 0, 2] = p0 * p2 + s * p1
    R[:, 1, 0] = p1 * p0 + s * p2
    R[:, 1, 1] = p1 * p1 + diag
    R[:, 1, 2] = p1 * p2 - s * p0
    R[:, 2, 0] = p2 * p0 - s * p1
    R[:, 2, 1] = p2 * p1 + s * p0
    R[:, 2, 2] = p2 * p2 + diag
    return 2.0 * R


def blob_positions(locations, quaternions, shell):
    """r = R(q) r_ref + x for every body (body/body.py:64-78), shape (Nb*nb, 3)."""
    R = rotation_matrices(quaternions)
    r = np.einsum("bij,kj->bki", R, shell) + np.asarray(locations)[:, None, :]
    return r.reshape(-1, 3)


def place_bodies(rng, nb, min_dist, xy_max, z_lo, z_hi, max_tries=200):
    """Rejection-sample nb centres with pairwise distance > min_dist using a
    cell list (x,y ~ U[0, xy_max], z ~ U[z_lo, z_hi])."""
    cell = min_dist
    grid = {}
    out = np.empty((nb, 3))
    k = 0
    tries = 0
    while k < nb:
        tries += 1
        if tries > max_tries * nb:
            raise RuntimeError("body placement failed: packing too dense")
        c = np.array([rng.uniform(0, xy_max), rng.uniform(0, xy_max), rng.uniform(z_lo, z_hi)])
        key = tuple((c // cell).astype(int))
        ok = True
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dz in (-1, 0, 1):
                    for idx in grid.get((key[0] + dx, key[1] + dy, key[2] + dz), ()):
                        if np.linalg.norm(out[idx] - c) <= min_dist:
                            ok = False
                            break
                    if not ok:
                        break
                if not ok:
                    break
            if not ok:
                break
        if ok:
            out[k] = c
            grid.setdefault(key, []).append(k)
            k += 1
    return out


class Suspension:
    """Bodies of one shell type: locations (Nb,3), quaternions (Nb,4), shell (nb,3)."""

    def __init__(self, locations, quaternions, shell, a, eta=1.0, name=""):
        self.locations = np.ascontiguousarray(locations, dtype=np.float64)
        self.quaternions = np.ascontiguousarray(quaternions, dtype=np.float64)
        self.shell = np.ascontiguousarray(shell, dtype=np.float64)
        self.a = float(a)
        self.eta = float(eta)
        self.name = name

    @property
    def n_bodies(self):
        return self.locations.shape[0]

    @property
    def blobs_per_body(self):
        return self.shell.shape[0]

    @property
    def n_blobs(self):
        return self.n_bodies * self.blobs_per_body

    def r_vectors(self):
        return blob_positions(self.locations, self.quaternions, self.shell)


def shells(n_bodies, shell, seed, xy_max, z_lo, z_hi, eta=1.0, name="", a=None):
    rng = np.random.default_rng(seed)
    R = np.linalg.norm(shell[0])
    a = blob_radius_of(shell) if a is None else a
    locs = place_bodies(rng, n_bodies, 2 * R + 2 * a, xy_max, z_lo, z_hi)
    quats = random_quaternions(rng, n_bodies)
    return Suspension(locs, quats, shell, a, eta, name)


def blobs_wall_matvec(n=2048, seed=0):
    """Free blobs for the plain M.F workload: returns (r, force, eta, a)."""
    rng = np.random.default_rng(seed)
    a = 0.5
    r = np.empty((n, 3))
    r[:, 0:2] = rng.uniform(0.0, 64 * a, (n, 2))
    r[:, 2] = rng.uniform(1.5 * a, 10 * a, n)
    f = rng.standard_normal((n, 3))
    return r, f, 1.0, a


def shells_42_256(seed=1, n_bodies=256):
    R = R42
    return shells(n_bodies, icosphere_42(R), seed, 60 * R, 1.2 * R, 5 * R, name="shells_42_%d" % n_bodies)


def shells_12_1024(seed=2, n_bodies=1024):
    R = 1.0
    shell = icosahedron(R)
    # blob radius 0.4 as the workload specifies (slightly below half the edge, 0.5257)
    side = 60 * R * np.sqrt(n_bodies / 256.0)
    return shells(n_bodies, shell, seed, side, 1.2 * R, 5 * R, name="shells_12_%d" % n_bodies, a=0.4)


def shells_42_4096(seed=4, n_bodies=4096, area_fraction=0.3):
    R = R42
    side = np.sqrt(n_bodies * np.pi * R * R / area_fraction)
    return shells(n_bodies, icosphere_42(R), seed, side, 1.1 * R, 3 * R, name="shells_42_%d" % n_bodies)


def shells_42_batch(seed=3, n_suspensions=64, lo=16, hi=512):
    """Independent suspensions of uneven size (list of Suspension)."""
    rng = np.random.default_rng(seed)
    counts = rng.integers(lo, hi + 1, size=n_suspensions)
    out = []
    R = R42
    for k, c in enumerate(counts):
        side = 60 * R * np.sqrt(max(int(c), 256) / 256.0)
        out.append(shells(int(c), icosphere_42(R), seed * 1000 + k, side, 1.2 * R, 5 * R,
                          name="batch_%d_%d" % (k, c)))
    return out
