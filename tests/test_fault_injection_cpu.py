"""Host-side fault injection: malformed scenes and BVHs are rejected by
mt_create with MT_ERR_INVALID before any CUDA call (so these run without a GPU),
and the message names what is wrong.  The reference builds its BVHs itself
(src/Scene/BVH.cpp:117-282) and trusts them; the drop-in boundary also accepts
prebuilt ones, so it checks them before the traversal can read past an array
or overflow its stack."""
import ctypes as C
import copy

import numpy as np
import pytest

import mitrace_gb300 as mt
from mitrace_gb300 import _abi as A
from oracle import oracle_py as orc

LEAF = A.MT_BVH_LEAF_BIT


def sphere_scene():
    """One 64-triangle sphere (above the 32-triangle BVH threshold) with the
    reference BVH attached, plus the box room's light and camera."""
    scene, cfg = mt.box_room(width=8, height=8, samples=1)
    m = mt.scenes.uv_sphere(0.4, segments=8, rings=4)
    nodes, idx = orc.bvh_build(m.positions.reshape(-1, 9).reshape(-1, 3, 3))
    m.bvh_nodes, m.bvh_indices = nodes, idx
    scene.meshes = [m]
    scene.instances = [mt.InstanceData(0, 0)]
    return scene, cfg


def create(scene, cfg):
    h = C.c_void_p()
    rc = A.lib.mt_create(mt.PackedScene(scene).ptr(), C.byref(cfg), C.byref(h))
    if rc == A.MT_OK:
        A.lib.mt_destroy(h)
    return rc, A.lib.mt_last_error().decode()


def corrupt(fn):
    scene, cfg = sphere_scene()
    m = scene.meshes[0]
    m.bvh_nodes = m.bvh_nodes.copy()
    m.bvh_indices = m.bvh_indices.copy()
    fn(m)
    return create(scene, cfg)


def first_inner(nodes):
    return next(i for i in range(nodes.shape[0]) if i != 1 and not nodes[i, 6] & LEAF)


def first_leaf(nodes):
    return next(i for i in range(nodes.shape[0]) if i != 1 and nodes[i, 6] & LEAF)


def test_valid_prebuilt_bvh_passes_validation():
    # on a box without a GPU the call gets past validation and fails at the
    # device (MT_ERR_CUDA); with one it succeeds
    rc, msg = create(*sphere_scene())
    assert rc in (A.MT_OK, A.MT_ERR_CUDA), msg


def test_child_index_out_of_range():
    def f(m):
        i = first_inner(m.bvh_nodes)
        m.bvh_nodes[i, 6] = m.bvh_nodes.shape[0] + 5
        m.bvh_nodes[i, 7] = m.bvh_nodes.shape[0] + 6
    rc, msg = corrupt(f)
    assert rc == A.MT_ERR_INVALID and "out of range" in msg


def test_leaf_range_past_the_index_array():
    def f(m):
        i = first_leaf(m.bvh_nodes)
        m.bvh_nodes[i, 7] = m.bvh_indices.shape[0] + 1
    rc, msg = corrupt(f)
    assert rc == A.MT_ERR_INVALID and "leaf range" in msg


def test_index_names_a_missing_triangle():
    def f(m):
        m.bvh_indices[0] = m.num_triangles
    rc, msg = corrupt(f)
    assert rc == A.MT_ERR_INVALID and "missing triangle" in msg


def test_siblings_not_adjacent():
    def f(m):
        i = first_inner(m.bvh_nodes)
        m.bvh_nodes[i, 7] = m.bvh_nodes[i, 6] + 2
    rc, msg = corrupt(f)
    assert rc == A.MT_ERR_INVALID and "adjacent" in msg


def test_cyclic_bvh():
    def f(m):
        i = first_inner(m.bvh_nodes)
        m.bvh_nodes[i, 6], m.bvh_nodes[i, 7] = 0, 1  # back to the root
    rc, msg = corrupt(f)
    assert rc == A.MT_ERR_INVALID


def test_bvh_deeper_than_the_traversal_stack():
    """A chain of 70 inner nodes (each with one leaf child) is well formed but
    deeper than the 64-entry traversal stack allows."""
    depth = 70
    scene, cfg = sphere_scene()
    m = scene.meshes[0]
    T = m.num_triangles
    nodes = np.zeros((2 * depth + 2, 8), np.uint32)
    lo = np.float32([-1, -1, -1]).view(np.uint32)
    hi = np.float32([1, 1, 1]).view(np.uint32)
    nodes[:, 0:3], nodes[:, 3:6] = lo, hi
    for k in range(depth):
        node = 0 if k == 0 else 2 * k + 1
        a = 2 * k + 2
        nodes[node, 6], nodes[node, 7] = a, a + 1
        nodes[a, 6], nodes[a, 7] = LEAF | 0, 1  # leaf: triangle index 0
    last = 2 * depth + 1
    nodes[last, 6], nodes[last, 7] = LEAF | 0, T
    m.bvh_nodes = nodes
    m.bvh_indices = np.arange(T, dtype=np.uint32)
    rc, msg = create(scene, cfg)
    assert rc == A.MT_ERR_INVALID and "depth" in msg


@pytest.mark.parametrize("what", ["material_texture", "negative_texture", "instance_mesh", "instance_material",
                                  "light_type", "env", "texture_empty", "no_positions"])
def test_scene_references(what):
    scene, cfg = mt.box_room(width=8, height=8, samples=1)
    scene = copy.deepcopy(scene)
    if what == "material_texture":
        scene.materials[0].base_tex = 3
    elif what == "negative_texture":
        scene.materials[0].normal_tex = -4
    elif what == "instance_mesh":
        scene.instances[0].mesh = len(scene.meshes)
    elif what == "instance_material":
        scene.instances[0].material = len(scene.materials) + 2
    elif what == "light_type":
        scene.lights[0].type = 9
    elif what == "env":
        scene.env = 0  # no textures
    elif what == "texture_empty":
        scene.textures.append(mt.TextureData(rgb8=np.zeros((0, 4, 3), np.uint8)))
    elif what == "no_positions":
        scene.meshes[0].positions = np.zeros((0, 3, 3), np.float32)
        scene.meshes[0].normals = np.zeros((0, 3, 3), np.float32)
    rc, msg = create(scene, cfg)
    assert rc == A.MT_ERR_INVALID, (what, rc, msg)
    assert msg
