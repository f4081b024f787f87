"""mscomplex_gb300 -- GB300-native (sm_103a) grid Morse-Smale complex.

The compute path is libdmsc.so (CUDA, built in-tree by ``build.build()``);
this package is its host-side mirror of the reference interfaces
(GridDataset / GridMSComplex / GridDataManager of nithins/mscomplex).
"""
from ._native import DmscError, load
from .dataset import Context, GridBatch, GridDataManager, GridDataset, GridMSComplex, GridServer, default_context

__all__ = ["DmscError", "load", "Context", "GridBatch", "GridDataManager", "GridDataset", "GridMSComplex", "GridServer", "default_context"]
