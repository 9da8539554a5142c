"""covertreex_gb300 — GB300 (sm_103a) engine for covertreex's residual-correlation
cover-tree kNN, behind the reference's ``cover_tree`` / engine API (``engine="cuda"``)."""
from .engine import CoverTree, CudaEngine, TreeEngine, build_tree, get_engine
from .factory import BuiltCoverTree, cover_tree
from .kernels import RBF, Kernel, Matern52
from .residual import ResidualCorrHostData, build_residual_backend

__all__ = ["cover_tree", "BuiltCoverTree", "CoverTree", "CudaEngine", "TreeEngine", "build_tree", "get_engine",
           "RBF", "Matern52", "Kernel", "ResidualCorrHostData", "build_residual_backend"]
