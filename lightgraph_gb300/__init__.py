"""lightgraph_gb300 -- GB300-native (sm_103a) LightGraph multiple-scattering path.

The compute runs in the in-tree CUDA library built by ``lightgraph_gb300.build``
and reached through the C ABI in include/lightgraph_c.h. This package mirrors
the reference's LightGraph / ScatterGrid / VolumeRender interface on top of it.
"""
from .lightgraph import (ColorRamp, Context, Films, Grid, Light, LightGraph, SceneSettings, ScatterGrid,  # noqa: F401
                         Shader, VolumeRender)
from ._capi import LightGraphError  # noqa: F401

__all__ = ["ColorRamp", "Context", "Films", "Grid", "Light", "LightGraph", "LightGraphError", "SceneSettings",
           "ScatterGrid", "Shader", "VolumeRender"]
