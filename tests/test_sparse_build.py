"""The library's sparse distance-volume build against a direct restatement of
the reference's DistanceVolumeBuilder.buildSparse (Scene/SDFModel.swift:256-355,
with sampleBrick / samplePosition / sampleField / combine at :357-570).

`dk_build_sparse_sphere_volume` skips bricks whose stored samples provably lie
outside the narrow band without sampling them (interval bounds of the union
chain).  The restatement below samples every brick, exactly as buildSparse
does, and keeps those whose stored samples meet the band; the two must keep the
same bricks in the same order with the same stored samples, bit for bit.  Runs
on the CPU (the host build; the GPU bake is checked against the host build in
test_sdf_bake.py).
"""
import numpy as np
import pytest

from denrimrendererkit_gb300 import library

F32 = np.float32
FLT_MAX = np.finfo(np.float32).max


def sample_field(spheres, x, y, z):
    """sampleField (SDFModel.swift:466-498) for sphere unions, in float32:
    returns distance, material, secondary material, blend per sample."""
    n = x.size
    dist = np.full(n, FLT_MAX, F32)
    mat = np.full(n, spheres[0]["material"], np.uint32)   # fallback: the first primitive's material
    sec = mat.copy()
    blend = np.zeros(n, F32)
    with np.errstate(over="ignore", invalid="ignore"):
        for s in spheres:
            cx, cy, cz = (F32(c) for c in s["center"])
            lx, ly, lz = x - cx, y - cy, z - cz
            d = np.sqrt((lx * lx + ly * ly) + lz * lz) - F32(s["radius"])   # simd_length(local) - radius
            m = np.uint32(s["material"])
            radius = max(F32(s.get("smooth_union_radius", 0.0)), F32(0))
            finite = np.isfinite(dist)
            if not radius > F32(1e-6):                      # combine: hard union
                take = ~finite | (d < dist)
                dist = np.where(take, d, dist)
                mat = np.where(take, m, mat)
                sec = np.where(take, m, sec)
                blend = np.where(take, F32(0), blend)
                continue
            h = np.clip(F32(0.5) + F32(0.5) * (d - dist) / radius, F32(0), F32(1)).astype(F32)
            nd = (d + (dist - d) * h) - radius * h * (F32(1) - h)   # mix(cand, cur, h) - r h (1 - h)
            w = F32(1) - h
            keep_cur = finite & (w <= F32(0.001))
            take = ~finite | (w >= F32(0.999))
            mix = finite & ~keep_cur & ~take
            new_dist = np.where(~finite, d, nd)
            new_mat = np.where(take, m, mat)
            new_sec = np.where(take | mix, m, sec)
            new_blend = np.where(take, F32(0), np.where(mix, w, blend))
            dist, mat, sec, blend = new_dist.astype(F32), new_mat, new_sec, new_blend.astype(F32)
    return dist, mat, sec, blend


def build_sparse(spheres, dims, bmin, bmax, brick, band):
    """buildSparse: bricks in z-y-x order, 2-sample stored overlap, kept when
    min <= band and max >= -band over the stored samples."""
    dims = [int(d) for d in dims]
    bmin = np.array(bmin, F32)
    ext = np.array(bmax, F32) - bmin
    out = []
    for oz in range(0, dims[2], brick[2]):
        for oy in range(0, dims[1], brick[1]):
            for ox in range(0, dims[0], brick[0]):
                origin = (ox, oy, oz)
                bd = [min(brick[a], dims[a] - origin[a]) for a in range(3)]
                so = [max(origin[a] - 2, 0) for a in range(3)]
                se = [min(origin[a] + bd[a] + 2, dims[a]) for a in range(3)]
                sd = [se[a] - so[a] for a in range(3)]
                idx = [np.arange(so[a], se[a]) for a in range(3)]
                # samplePosition: boundsMin + extent * (i / (n - 1)), float32 throughout
                pos = [bmin[a] + ext[a] * (idx[a].astype(F32) / F32(dims[a] - 1)) for a in range(3)]
                zz, yy, xx = np.meshgrid(pos[2], pos[1], pos[0], indexing="ij")   # index x + y*w + z*w*h
                d, m, s2, b = sample_field(spheres, xx.ravel(), yy.ravel(), zz.ravel())
                if d.min() <= F32(band) and d.max() >= -F32(band):
                    out.append(dict(origin=tuple(so), dims=tuple(sd), core=origin, distance=d, material_a=m,
                                    material_b=s2, blend=b))
    return out


def spheres_seeded(seed, count, smooth):
    rng = np.random.default_rng(seed)
    return [dict(center=tuple(float(v) for v in rng.uniform(-0.6, 0.6, 3)), radius=float(rng.uniform(0.08, 0.3)),
                 material=int(rng.integers(0, 3)), smooth_union_radius=smooth) for _ in range(count)]


CASES = [
    # (spheres, resolution, brick size, narrow band)
    (spheres_seeded(1, 6, 0.05), (24, 24, 24), (8, 8, 8), 0.08),         # smooth union, even bricks
    (spheres_seeded(2, 5, 0.0), (21, 19, 23), (5, 6, 4), 0.12),          # hard union, ragged edges
    (spheres_seeded(3, 9, 0.1), (33, 17, 29), (7, 7, 7), 0.05),          # wide smoothing, thin band
    ([dict(center=(0.0, 0.0, 0.0), radius=0.55, material=0)], (20, 20, 20), (5, 5, 5), 0.3),  # RenderSessionTests
]


@pytest.mark.parametrize("fp16", [False, True], ids=["fp32", "fp16"])
@pytest.mark.parametrize("spheres,res,brick,band", CASES)
def test_host_build_keeps_the_bricks_and_samples_of_build_sparse(dk_lib, spheres, res, brick, band, fp16):
    # fp16: the same bricks (selected on the exact samples, as buildSparse
    # does), every stored distance rounded to half precision.
    want = build_sparse(spheres, res, (-1, -1, -1), (1, 1, 1), brick, band)
    if fp16:
        for w in want:
            w["distance"] = w["distance"].astype(np.float16).astype(np.float32)
    vol = library.SparseVolume(spheres, res, (-1, -1, -1), (1, 1, 1), brick, band, on_device=False,
                               fp16_distances=fp16)
    assert len(vol.bricks) == len(want) > 0
    total = sum(int(np.prod(w["dims"])) for w in want)
    assert len(vol.samples) == total
    for k, w in enumerate(want):
        b = vol.bricks[k]
        assert tuple(int(v) for v in b["grid_origin_and_volume"][:3]) == w["origin"]
        dims_off = b["dimensions_and_sample_offset"]
        assert tuple(int(v) for v in dims_off[:3]) == w["dims"]
        off, n = int(dims_off[3]), int(np.prod(w["dims"]))
        got = vol.samples[off:off + n]
        assert np.array_equal(got["distance"].view(np.uint32), w["distance"].view(np.uint32)), k
        assert np.array_equal(got["material_a"], w["material_a"]), k
        assert np.array_equal(got["material_b"], w["material_b"]), k
        assert np.array_equal(got["material_blend"].view(np.uint32), w["blend"].view(np.uint32)), k
        # the descriptor's distance range is the stored samples' range
        assert b["sample_bounds_min"][3] == w["distance"].min() and b["sample_bounds_max"][3] == w["distance"].max()
    # the brick grid points each kept brick's cell at its index and marks the rest empty
    grid = vol.grids[0]
    gdim = [int(v) for v in grid["dimensions_and_index_offset"][:3]]
    cells = gdim[0] * gdim[1] * gdim[2]
    index = vol.grid_indices[:cells]
    kept = {tuple(w["core"][a] // brick[a] for a in range(3)): k for k, w in enumerate(want)}
    for cz in range(gdim[2]):
        for cy in range(gdim[1]):
            for cx in range(gdim[0]):
                v = int(index[cx + cy * gdim[0] + cz * gdim[0] * gdim[1]])
                assert v == kept.get((cx, cy, cz), 0xFFFFFFFF)


def test_restatement_drops_bricks_outside_the_band():
    # The restatement itself: a band that no sample reaches keeps nothing.
    s = [dict(center=(0.0, 0.0, 0.0), radius=0.2, material=0)]
    assert build_sparse(s, (16, 16, 16), (-1, -1, -1), (1, 1, 1), (4, 4, 4), 0.05)
    far = [dict(center=(5.0, 5.0, 5.0), radius=0.2, material=0)]
    assert not build_sparse(far, (16, 16, 16), (-1, -1, -1), (1, 1, 1), (4, 4, 4), 0.05)
