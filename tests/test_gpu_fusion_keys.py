"""Fusion with a voxel whose key equals the hash table's empty-slot marker.

The reference's voxel key (patchmatch_stereo.cpp:1045-1046) is
(vx*73856093) ^ (vy*19349663) ^ (vz*83492791) in 64 bits, so a real voxel can
have any key -- including the 0x7F7F7F7F7F7F7F7F pattern the device hash table
clears its slots with.  The reference's unordered_map is unaffected; the
device table must be too: that voxel may neither claim a slot that still
reads as empty nor absorb a later voxel probing the same slot.  The case is
built exactly: voxel (6368544320783, 168820, 0) has the marker key, and voxel
(167396, 0, 0) hashes to the marker's home slot in a table of 2^21 slots
(three 512x512 maps).  Each map holds one valid pixel at its principal point
(ray = (0, 0, 1), so the world point is exactly -t for R = I), the marker
voxel first in the point order and the colliding one last.  The cloud must
equal the oracle's."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

M64 = (1 << 64) - 1
KA, KB, KC = 73856093, 19349663, 83492791
EMPTY = 0x7F7F7F7F7F7F7F7F
SENTINEL_VOXEL = (6368544320783, 168820, 0)
COLLIDER_VOXEL = (167396, 0, 0)
OTHER_VOXEL = (-4000, 2500, 0)
SIDE = 512  # 3 maps of 512 x 512: 2^21 table slots


def voxel_key(v):
    return ((v[0] * KA) & M64) ^ ((v[1] * KB) & M64) ^ ((v[2] * KC) & M64)


def hash64(x):
    """The device table's slot hash (the 64-bit finaliser of MurmurHash3)."""
    x ^= x >> 33
    x = (x * 0xFF51AFD7ED558CCD) & M64
    x ^= x >> 33
    x = (x * 0xC4CEB9FE1A85EC53) & M64
    x ^= x >> 33
    return x


@pytest.fixture(scope="module")
def mvs():
    import recon_mvs

    recon_mvs.load_library()
    return recon_mvs


def one_point_map(px, py, voxel, vsize):
    """A map whose only valid pixel (px, py) back-projects to the centre of
    `voxel` (depth 1, R = I, principal point at the pixel centre)."""
    depth = np.full((SIDE, SIDE), np.nan, np.float32)
    depth[py, px] = 1.0
    support = np.full((SIDE, SIDE), 5, np.uint8)
    conf = np.ones((SIDE, SIDE), np.float32)
    P = [(voxel[0] + 0.5) * vsize, (voxel[1] + 0.5) * vsize, (voxel[2] + 0.5) * vsize]
    pose = np.zeros(13)
    pose[[0, 4, 8]] = 1.0
    pose[9:12] = [-P[0], -P[1], 1.0 - P[2]]
    intr = [500.0, 500.0, px + 0.5, py + 0.5, 0, 0, 0, 0, 0, SIDE, SIDE]
    return (depth, support, conf), pose, intr


def test_voxel_with_the_empty_marker_key(mvs):
    assert voxel_key(SENTINEL_VOXEL) == EMPTY
    mask = (1 << 21) - 1
    assert hash64(voxel_key(COLLIDER_VOXEL)) & mask == hash64(EMPTY) & mask
    vsize = 0.001
    specs = [(0, 0, SENTINEL_VOXEL), (200, 300, OTHER_VOXEL), (SIDE - 1, SIDE - 1, COLLIDER_VOXEL)]
    maps, poses, intr = [], [], []
    for px, py, v in specs:
        m, p, k = one_point_map(px, py, v, vsize)
        maps.append(m)
        poses.append(p)
        intr.append(k)
    cfg_o = O.make_config(fusion_voxel_size_m=vsize)
    want_pos, want_nrm, want_conf = O.fuse_depth_maps("oracle", maps, poses, intr, cfg_o)
    assert len(want_pos) == 3
    cfg = mvs.MvsConfig(fusion_voxel_size_m=vsize)
    pc = mvs.FuseDepthMaps([mvs.DepthMap(*m) for m in maps], poses, intr, cfg)
    order = np.lexsort((pc.positions[:, 2], pc.positions[:, 1], pc.positions[:, 0]))
    assert len(order) == 3, "a voxel was merged into the one with the empty-marker key"
    assert np.array_equal(pc.positions[order], want_pos)
    assert np.array_equal(pc.normals[order], want_nrm)
    assert np.array_equal(pc.confidences[order], want_conf)
    assert sorted(pc.counts.tolist()) == [1, 1, 1]
    assert EMPTY in {int(k) & M64 for k in pc.keys}
