"""Material.gpu_material against the reference's packing tests
(Tests/DenrimRendererKitTests/APITests.swift:2140-2250), restated.

* testMaterialSpecularClearcoatSheenAndIORReachGPUParameters: every layered-BSDF
  control lands in the GPUMaterial slot the shader reads.
* testMaterialTransmissionDefaultsInheritBaseSurfaceControls: an unset
  transmission colour, roughness and IOR inherit the base surface's.
"""
import numpy as np
import pytest

from denrimrendererkit_gb300.scene import Material

ACC = 1e-4


def test_specular_clearcoat_sheen_and_ior_reach_gpu_parameters():
    m = Material(
        base_color=(0.8, 0.7, 0.6), roughness=0.35, metallic=0.2, specular=0.6, specular_color=(0.9, 0.7, 0.5),
        index_of_refraction=1.8, specular_anisotropy=0.65, clearcoat=0.4, clearcoat_color=(0.25, 0.8, 0.9),
        clearcoat_attenuation_color=(0.5, 0.65, 0.8), clearcoat_thickness=0.6, clearcoat_roughness=0.08,
        clearcoat_index_of_refraction=1.6, thin_film=0.8, thin_film_thickness_nanometers=520,
        thin_film_index_of_refraction=1.42, sheen=0.55, sheen_color=(0.3, 0.4, 0.5), sheen_roughness=0.7,
        subsurface=0.8, subsurface_color=(0.95, 0.42, 0.28), subsurface_radius=(1.2, 0.45, 0.25),
        subsurface_scale=0.32, subsurface_anisotropy=0.18, transmission=0.75, transmission_color=(0.2, 0.6, 0.9),
        transmission_roughness=0.18, transmission_index_of_refraction=1.33,
        transmission_absorption_color=(0.5, 0.75, 0.95), transmission_absorption_distance=1.25, thin_walled=True,
        volume_scattering=0.7, volume_scattering_color=(0.8, 0.85, 0.9), volume_scattering_distance=0.6,
        volume_anisotropy=0.22)
    g = m.gpu_material()
    want = {
        ("parameters", 0): 0.35, ("parameters", 1): 0.2,
        ("parameters2", 0): 0.6, ("parameters2", 1): 1.8, ("parameters2", 2): 0.4, ("parameters2", 3): 0.08,
        ("specular_color", 0): 0.9, ("specular_color", 1): 0.7, ("specular_color", 2): 0.5,
        ("specular_color", 3): 1.6,
        ("sheen_color", 0): 0.3, ("sheen_color", 1): 0.4, ("sheen_color", 2): 0.5, ("sheen_color", 3): 0.55,
        ("transmission_color", 0): 0.2, ("transmission_color", 1): 0.6, ("transmission_color", 2): 0.9,
        ("transmission_color", 3): 1.0,
        ("parameters3", 0): 0.7, ("parameters3", 1): 0.18, ("parameters3", 2): 1.33, ("parameters3", 3): 0.65,
        ("clearcoat_color", 0): 0.25, ("clearcoat_color", 1): 0.8, ("clearcoat_color", 2): 0.9,
        ("clearcoat_color", 3): 0.0,
        ("clearcoat_attenuation", 0): 0.5, ("clearcoat_attenuation", 1): 0.65, ("clearcoat_attenuation", 2): 0.8,
        ("clearcoat_attenuation", 3): 0.6,
        ("transmission_absorption", 0): 0.5, ("transmission_absorption", 1): 0.75,
        ("transmission_absorption", 2): 0.95, ("transmission_absorption", 3): 1.25,
        ("thin_film", 0): 0.8, ("thin_film", 1): 520.0, ("thin_film", 2): 1.42,
        ("subsurface_color", 0): 0.95, ("subsurface_color", 1): 0.42, ("subsurface_color", 2): 0.28,
        ("subsurface_color", 3): 0.8,
        ("subsurface_radius", 0): 1.2, ("subsurface_radius", 1): 0.45, ("subsurface_radius", 2): 0.25,
        ("subsurface_radius", 3): 0.32,
        ("subsurface_parameters", 0): 0.18,
        ("volume_scattering", 0): 0.8, ("volume_scattering", 1): 0.85, ("volume_scattering", 2): 0.9,
        ("volume_scattering", 3): 0.7,
        ("volume_parameters", 0): 0.6, ("volume_parameters", 1): 0.22,
        ("emission", 3): 0.75,
    }
    for (field, lane), value in want.items():
        assert float(g[field][lane]) == pytest.approx(value, abs=ACC), (field, lane)


def test_transmission_defaults_inherit_base_surface_controls():
    m = Material(base_color=(0.35, 0.6, 0.9), roughness=0.42, index_of_refraction=1.47, transmission=1)
    g = m.gpu_material()
    np.testing.assert_allclose(g["transmission_color"][:3], (0.35, 0.6, 0.9), atol=ACC)
    assert float(g["parameters3"][1]) == pytest.approx(0.42, abs=ACC)   # transmissionRoughness
    assert float(g["parameters3"][2]) == pytest.approx(1.47, abs=ACC)   # transmissionIndexOfRefraction
    assert float(g["transmission_color"][3]) == 0.0                      # thinWalled false
    assert float(g["emission"][3]) == 1.0                                # transmission weight
