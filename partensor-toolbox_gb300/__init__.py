"""partensor-toolbox_gb300: GB300-native CPD-ALS hot path behind Partensor's cpd /
cpdDimTree / gtc interface.

The directory name carries a hyphen, so it is imported as ``partensor_toolbox_gb300``
through ``load_package()`` of the repository's ``__graft_entry__.py`` (or any
importlib.util.spec_from_file_location call on this file).  Compute entry points live in
``cpd`` and call libptg.so (built by ``build.py``); importing them without the library
raises.
"""
from . import _lib  # noqa: F401
from .cpd import (CONSTANT, NONNEGATIVITY, ORTHOGONALITY, SPARSITY, UNCONSTRAINED, Context,  # noqa: F401
                  Options, Status, Tensor, WarmStartModel, cpd, cpd_batched, cpd_file, cpd_resident, cpdDimTree,
                  default_context, mttkrp, write_factor_file, write_tensor_file)
from .gtc import SparseOptions, SparseStatus, gtc, gtc_coo, gtc_device, gtc_stochastic  # noqa: F401
from .gtc import sort_mode as gtc_sort_mode  # noqa: F401
from ._lib import PtgError  # noqa: F401
from . import datagen  # noqa: F401
