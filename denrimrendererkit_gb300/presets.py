"""Built-in material presets used by the serving workload.

The parameters restate BuiltInMaterialLibrary.presets
(Sources/DenrimRendererKit/Scene/BuiltInMaterialLibrary.swift:60-350) for the
families a material-preview job draws from: diffuse, plastic, fabric (sheen),
subsurface, metal and coating (clearcoat, and the thin-film coating).
"""
from __future__ import annotations

from .scene import Material

PRESETS = {
    # .diffuse
    "matte.clay": Material(base_color=(0.78, 0.62, 0.48), roughness=0.82, specular=0.25),
    "matte.paper": Material(base_color=(0.92, 0.9, 0.86), roughness=0.9, specular=0.18),
    "matte.charcoal": Material(base_color=(0.025, 0.025, 0.023), roughness=0.86, specular=0.12),
    # .plastic
    "plastic.soft-black": Material(base_color=(0.035, 0.034, 0.032), roughness=0.38, specular=0.55, clearcoat=0.18,
                                   clearcoat_roughness=0.24),
    "plastic.gloss-white": Material(base_color=(0.86, 0.86, 0.82), roughness=0.18, specular=0.7, clearcoat=0.45,
                                    clearcoat_roughness=0.08),
    "rubber.black": Material(base_color=(0.012, 0.012, 0.011), roughness=0.78, specular=0.22),
    # .fabric
    "fabric.velvet-purple": Material(base_color=(0.22, 0.08, 0.42), roughness=0.74, specular=0.18, sheen=0.72,
                                     sheen_color=(0.72, 0.52, 1.0), sheen_roughness=0.82),
    "fabric.denim-blue": Material(base_color=(0.055, 0.12, 0.26), roughness=0.88, specular=0.16, sheen=0.3,
                                  sheen_color=(0.35, 0.5, 0.78), sheen_roughness=0.9),
    # .subsurface
    "subsurface.skin-warm": Material(base_color=(0.82, 0.52, 0.38), roughness=0.56, specular=0.38,
                                     index_of_refraction=1.38, subsurface=0.82, subsurface_color=(0.95, 0.48, 0.32),
                                     subsurface_radius=(1.0, 0.42, 0.24), subsurface_scale=0.34,
                                     subsurface_anisotropy=0.18),
    "subsurface.wax-cream": Material(base_color=(0.94, 0.82, 0.58), roughness=0.48, specular=0.42,
                                     index_of_refraction=1.44, subsurface=0.88, subsurface_color=(0.98, 0.82, 0.48),
                                     subsurface_radius=(1.3, 0.88, 0.42), subsurface_scale=0.48,
                                     subsurface_anisotropy=0.0),
    "subsurface.jade-green": Material(base_color=(0.28, 0.62, 0.48), roughness=0.42, specular=0.48,
                                      index_of_refraction=1.56, clearcoat=0.14, clearcoat_roughness=0.16,
                                      subsurface=0.7, subsurface_color=(0.38, 0.86, 0.58),
                                      subsurface_radius=(0.38, 0.9, 0.52), subsurface_scale=0.24,
                                      subsurface_anisotropy=0.08),
    # .metal
    "metal.chrome": Material(base_color=(0.95, 0.95, 0.93), roughness=0.012, metallic=1.0),
    "metal.aluminum": Material(base_color=(0.84, 0.85, 0.84), roughness=0.08, metallic=1.0),
    "metal.brushed-aluminum": Material(base_color=(0.84, 0.85, 0.84), roughness=0.16, metallic=1.0,
                                       specular_anisotropy=0.72),
    "metal.gold": Material(base_color=(1.0, 0.72, 0.29), roughness=0.06, metallic=1.0),
    "metal.copper": Material(base_color=(0.98, 0.45, 0.24), roughness=0.07, metallic=1.0),
    # .coating
    "coating.car-red": Material(base_color=(0.72, 0.025, 0.018), roughness=0.34, specular=0.55, clearcoat=0.9,
                                clearcoat_color=(1.0, 0.92, 0.88), clearcoat_roughness=0.045),
    "coating.pearl-white": Material(base_color=(0.86, 0.84, 0.78), roughness=0.28, specular=0.6, clearcoat=0.85,
                                    clearcoat_color=(1.0, 0.94, 0.82), clearcoat_roughness=0.04),
    "coating.iridescent-amber": Material(base_color=(0.88, 0.24, 0.035), roughness=0.18, specular=0.72,
                                         specular_color=(1.0, 0.9, 0.74), clearcoat=0.95,
                                         clearcoat_color=(1.0, 0.68, 0.2), clearcoat_roughness=0.035,
                                         clearcoat_index_of_refraction=1.55, thin_film=0.48,
                                         thin_film_thickness_nanometers=520.0, thin_film_index_of_refraction=1.38),
}

# The serving workload's seven families and the presets each draws from.
FAMILIES = {
    "diffuse": ("matte.clay", "matte.paper", "matte.charcoal"),
    "plastic": ("plastic.soft-black", "plastic.gloss-white", "rubber.black"),
    "sheen": ("fabric.velvet-purple", "fabric.denim-blue"),
    "subsurface": ("subsurface.skin-warm", "subsurface.wax-cream", "subsurface.jade-green"),
    "metal": ("metal.chrome", "metal.aluminum", "metal.brushed-aluminum", "metal.gold", "metal.copper"),
    "clearcoat": ("coating.car-red", "coating.pearl-white"),
    "thin-film": ("coating.iridescent-amber",),
}
