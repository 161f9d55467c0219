"""mapp4py_gb300: GB300-native EAM molecular dynamics and minimization with
the interface of MAPP's EAM path (mapp4py.md.atoms.ff_eam_*, md.nvt,
md.min_lbfgs, md.min_cg, ls_bt, ls_golden, ls_brent).  Compute runs in libmappg.so (CUDA, sm_103a) behind
the C ABI of include/mappg.h."""
from . import md  # noqa: F401
from .md import ls_brent, ls_bt, ls_golden  # noqa: F401

__all__ = ["md", "ls_bt", "ls_golden", "ls_brent"]
