"""Known-answer tests of the MDAO occupancy restatement (oracle), CPU only.

The reference voxelises spheres in GLSL (mdao_volume.geom.glsl / mdao_volume.frag.glsl) into an R8 texture
with additive blending; no reference output exists to pin it. These cases follow from the shader text:
  * volume size rule of SphereRenderer.cpp:2463-2476 (x rounded up to a multiple of 4, maxLod);
  * the fragment shader discards a voxel when its closest corner lies outside the sphere, before it tests
    for a sphere inside the voxel, so a small sphere inside one voxel contributes nothing;
  * a voxel whose farthest corner lies inside the sphere gets 1 (255 in R8);
  * R8 blending saturates: min(255, sum of rounded fragment values);
  * the R8 mip step divides by 8 always (edge attenuation), rounded half up."""
import numpy as np

import oracle


def test_mdao_dims():
    assert oracle.mdao_dims((0, 0, 0, 112, 112, 112), 128) == ((128, 128, 128), 128.0, 6.0)
    dims, shortest, max_lod = oracle.mdao_dims((0, 0, 0, 10, 5, 3), 64)
    assert dims == (64, 32, 20) and shortest == 20.0 and max_lod == 5.0
    # x is rounded up to a multiple of four, y and z to the next integer
    dims, _, _ = oracle.mdao_dims((0, 0, 0, 5, 10, 3), 64)
    assert dims == (32, 64, 20)
    dims, _, _ = oracle.mdao_dims((0, 0, 0, 3.3, 10, 1), 100)
    assert dims[0] % 4 == 0 and dims[0] >= 33 and dims[1:] == (100, 10)
    assert oracle.mdao_dims((0, 0, 0, 1, 1, 1), 100)[2] == 6.0  # ceil(log2 100) - 1


def test_small_sphere_inside_a_voxel_is_discarded():
    clip = (0, 0, 0, 8, 8, 8)
    dims, _, _ = oracle.mdao_dims(clip, 8)
    x = np.array([[2.5, 3.5, 4.5, 0.2], [5.5, 1.5, 6.5, 0.6]], np.float32)  # no voxel corner inside either
    for u8 in (True, False):
        assert not oracle.mdao_volume_f32(x, clip, dims, unorm8=u8).any()


def test_big_sphere_interior_is_full_and_volume_is_close():
    clip = (0, 0, 0, 16, 16, 16)
    dims, _, _ = oracle.mdao_dims(clip, 16)
    x = np.array([[8.0, 8.0, 8.0, 5.0]], np.float32)
    v8 = oracle.mdao_volume_f32(x, clip, dims, unorm8=True)
    vf = oracle.mdao_volume_f32(x, clip, dims, unorm8=False)
    assert v8[8, 8, 8] == 1.0 and vf[8, 8, 8] == 1.0
    assert v8[0, 0, 0] == 0.0
    true_volume = 4.0 / 3.0 * np.pi * 125.0
    assert abs(vf.sum() - true_volume) / true_volume < 0.08
    # one sphere: each voxel holds a single fragment, so R8 is the rounded fraction
    assert np.abs(v8 * 255.0 - np.rint(vf * 255.0)).max() <= 1.0
    assert np.all(np.abs(v8 - vf) <= 0.5 / 255.0 + 1e-7)
    # fractions are multiples of 1/27 or 1 (27-sample coverage)
    k = vf * 27.0
    assert np.allclose(k, np.rint(k), atol=1e-5)


def test_r8_blend_saturates_and_fp32_sums():
    clip = (0, 0, 0, 8, 8, 8)
    dims, _, _ = oracle.mdao_dims(clip, 8)
    one = np.array([[4.0, 4.0, 4.0, 1.2]], np.float32)
    v1 = oracle.mdao_volume_f32(one, clip, dims, unorm8=True)
    many = np.repeat(one, 10, axis=0)
    v10 = oracle.mdao_volume_f32(many, clip, dims, unorm8=True)
    expect = np.minimum(np.rint(v1 * 255.0) * 10, 255) / 255.0
    assert np.array_equal(v10, expect.astype(np.float32))
    f10 = oracle.mdao_volume_f32(many, clip, dims, unorm8=False)
    f1 = oracle.mdao_volume_f32(one, clip, dims, unorm8=False)
    assert np.allclose(f10, np.minimum(f1 * 10, 1.0), atol=1e-6)


def test_particles_outside_the_clip_box_are_clipped():
    """A point primitive is clipped by its centre: a sphere centred outside the box leaves no trace even
    where it overlaps the box."""
    clip = (0, 0, 0, 8, 8, 8)
    dims, _, _ = oracle.mdao_dims(clip, 8)
    x = np.array([[-0.5, 4.0, 4.0, 2.0], [4.0, 8.5, 4.0, 2.0]], np.float32)
    assert not oracle.mdao_volume_f32(x, clip, dims).any()
    inside = np.array([[0.5, 4.0, 4.0, 2.0]], np.float32)
    assert oracle.mdao_volume_f32(inside, clip, dims).any()


def test_r8_mip_step():
    k = np.full((4, 4, 4), 200, np.int64)
    lv = oracle.mdao_mip_u8((k / 255.0).astype(np.float32))
    assert lv.shape == (2, 2, 2) and np.all(np.rint(lv * 255) == 200)
    # a dimension of size one is attenuated by the /8 rule: 4 children of 200 -> (800 + 4) / 8 = 100
    thin = (np.full((1, 2, 2), 200) / 255.0).astype(np.float32)
    assert np.rint(oracle.mdao_mip_u8(thin) * 255).item() == 100
    # rounding half up: children summing to 4 (mod 8)
    src = np.zeros((2, 2, 2), np.float32)
    src[0, 0, 0] = 12 / 255.0
    assert np.rint(oracle.mdao_mip_u8(src) * 255).item() == 2
    src[0, 0, 0] = 11 / 255.0
    assert np.rint(oracle.mdao_mip_u8(src) * 255).item() == 1
