"""Mesh generators and Mesh.gpuTriangles packing against the reference's own
known answers (MeshTests.swift:7-68).  The loaders those tests also cover
(OBJ, PLY) sit above the boundary and are not part of this library."""
import numpy as np

from denrimrendererkit_gb300.scene import Mesh


def test_box_creates_twelve_triangles():
    # MeshTests.testBoxCreatesTwelveTriangles (:7-15)
    mesh = Mesh.box(size=(2, 4, 6))
    assert len(mesh.vertices) == 8 and len(mesh.indices) == 36
    assert len(mesh.gpu_triangles(0)) == 12
    assert mesh.vertices.min(axis=0).tolist() == [-1, -2, -3] and mesh.vertices.max(axis=0).tolist() == [1, 2, 3]


def test_gpu_triangles_carry_ids():
    # MeshTests.testGPUTrianglesCarryIDs (:17-32)
    tris = Mesh.quad((-1, -1, 0), (1, -1, 0), (1, 1, 0), (-1, 1, 0)).gpu_triangles(material_id=3, object_id=9)
    assert int(tris[0]["material_id"]) == 3 and int(tris[0]["object_id"]) == 9
    assert int(tris[0]["primitive_id"]) == 0 and int(tris[1]["primitive_id"]) == 1


def test_gpu_triangles_preserve_imported_vertex_normals():
    # MeshTests.testGPUTrianglesPreserveImportedVertexNormals (:34-54)
    mesh = Mesh(np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32), np.array([0, 1, 2], np.uint32),
                normals=np.array([[1, 0, 0], [0, 1, 0], [0, 0, 1]], np.float32))
    t = mesh.gpu_triangles(0)[0]
    assert t["n0"][:3].tolist() == [1, 0, 0] and t["n1"][:3].tolist() == [0, 1, 0] and t["n2"][:3].tolist() == [0, 0, 1]


def test_box_bounds_match_input_corners():
    # MeshTests.testBoxBoundsMatchInputCorners (:56-68)
    mesh = Mesh.box((-1, -2, -3), (4, 5, 6))
    assert mesh.vertices.min(axis=0).tolist() == [-1, -2, -3]
    assert mesh.vertices.max(axis=0).tolist() == [4, 5, 6]
