"""covertreex_gb300 — GB300 (sm_103a) engine for covertreex's residual-correlation
cover-tree kNN, behind the reference's ``cover_tree`` / ``CoverTree(runtime).fit`` /
engine API (``engine="cuda"``)."""
from .api import CoverTree, Residual, Runtime, configure_residual_correlation, get_residual_backend
from .engine import CoverTree as EngineCoverTree
from .engine import CudaEngine, TreeEngine, build_tree, get_engine
from .factory import BuiltCoverTree, cover_tree
from .kernels import RBF, Kernel, Matern52
from .residual import ResidualCorrHostData, build_residual_backend

__all__ = ["cover_tree", "BuiltCoverTree", "CoverTree", "Runtime", "Residual", "EngineCoverTree", "CudaEngine",
           "TreeEngine", "build_tree", "get_engine", "RBF", "Matern52", "Kernel", "ResidualCorrHostData",
           "build_residual_backend", "configure_residual_correlation", "get_residual_backend"]
