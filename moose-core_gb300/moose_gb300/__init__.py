"""GB300-native HSolve: MOOSE's Hines solver as hand-written sm_103a kernels.

Modules:
  abi      -- ctypes mirror of include/moose_gb300.h and the CellModel container
  models   -- seeded synthetic cells (HH cable, branched HH+Ca+K(Ca), SynChans)
  hsolve   -- HSolve: the one-cell drop-in (FP64, reference operation order)
  batch    -- Batch: thousands of cells in one persistent kernel
  swc, genesis, rdes -- model loaders: SWC files, GENESIS .p files, rdesigneur's
              cell prototypes and channel/passive distributions
  build    -- compiles libmoose_gb300.so in-tree
"""
from .abi import CellModel, HS_PREC_FP64, HS_PREC_MIXED  # noqa: F401
