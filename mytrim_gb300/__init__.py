"""mytrim_gb300 -- MyTRIM's binary-collision cascade engine on one GB300 GPU.

The compute path is libmytrim_gpu.so (CUDA for sm_103a, C ABI in
include/mytrim_gpu.h); this package is its Python front.
"""
from .engine import ElementSpec, Engine, LayerSpec, SimSpec, summarize
from .api import (Element, IonBase, MaterialBase, SampleBase, SampleLayers, SampleSolid, SimconfType,
                  TrimGPU, sampleClusters)

__all__ = ["Engine", "SimSpec", "LayerSpec", "ElementSpec", "summarize", "SimconfType", "Element",
           "MaterialBase", "SampleBase", "SampleSolid", "SampleLayers", "sampleClusters", "IonBase", "TrimGPU"]
