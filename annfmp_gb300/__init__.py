"""annfmp_gb300: annfmp's propagation-assisted k-d tree nearest-neighbour fields on one GB300 GPU.

Public API (mirrors the reference package ``annfmp``):
  ANNField                  facade, ``algorithm="gb300"`` (annfmp/base.py)
  ANNFieldPropKDTreeGB300   the pipeline estimator (annfmp/openmp/base.py)
  ANNFieldPropKDTreeOpenCLOPTGB300  the GPU backend's algorithm (annfmp/openclopt/base.py)
  KDTree                    the k-d tree estimator (annfmp/openmp/kdtree/base.py)
"""
__version__ = "0.1.0"

from .base import ANNField  # noqa: E402,F401
from .field import ANNFieldPropKDTreeGB300  # noqa: E402,F401
from .kdtree import KDTree  # noqa: E402,F401
from .openclopt import ANNFieldPropKDTreeOpenCLOPTGB300  # noqa: E402,F401
