"""Algorithmic byte counts for the roofline of the HSolve step kernels.

The unit is one compartment-step: one compartment advanced by one dt.  The
algorithmic bytes are the minimum DRAM traffic if every per-compartment
quantity the step needs were read once and every piece of state written once
per step, with rate tables and elimination temporaries on chip:

  V (FP64)                         read + write          16 B
  each gate state                  read + write          2 x state size
  each channel Gbar                read                  param size
  passive row: diag, off-diagonal,
      2C/dt, Em/Rm (FP64)          read                  32 B
  each Ca pool: c                  read + write          2 x state size
      factor1, factor2             read                  2 x param size
  each HHChannel2D: X              read + write          2 x state size
      Gbar                         read                  param size
  each SynChan: X, Y               read + write          4 x state size
      norm                         read                  param size

state/param size is 8 B in FP64 and 4 B in the mixed-precision path.  The
mixed kernel keeps each HH gate state as a two-float sum (8 B, so 16 B read
and written) for accuracy; the algorithmic count takes the FP32 state the
precision split calls for, so those 8 extra bytes per gate are overhead of
the design, visible in the measured DRAM traffic.
"""
import numpy as np

from .abi import HS_PREC_FP64


def bytes_per_cell_step(m, precision):
    s = 8 if precision == HS_PREC_FP64 else 4
    n = m.n_compt
    gates = int((m.chan_Xpower > 0).sum() + (m.chan_Ypower > 0).sum() + (m.chan_Zpower > 0).sum())
    total = 16 * n + 32 * n
    total += gates * 2 * s + len(m.chan_compt) * s
    total += len(m.pool_compt) * (2 * s + 2 * s)
    total += len(m.c2d_compt) * (2 * s + s)
    total += len(m.syn_compt) * (4 * s + s)
    return total


def algorithmic_bytes(cells, precision):
    """(total bytes per step over all cells, bytes per compartment-step)."""
    tot = sum(bytes_per_cell_step(m, precision) for m in cells)
    ncomp = sum(m.n_compt for m in cells)
    return tot, tot / max(1, ncomp)
