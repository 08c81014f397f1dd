"""GB300 (sm_103a) implementation of ttcode's implicit flux-limited-diffusion
radiation/gas energy step (COUPLED_ENERGY_EQS + SOLVE_WITH_SOR) behind a C ABI.

The compute lives in ``_lib/libttfld.so`` (CUDA, built by ``build.py``); this
package holds the host-side mirror of the reference interface (``fld``), the
grid metrics (``grid``), the seeded synthetic shells (``synthetic``), and the
reference's run files: the input file (``ipp``), restart and snapshot files
(``akttd``), opacity tables (``opacity``), read with Fortran's list-directed
rules (``fortio``).
"""
from .grid import Grid, gitter  # noqa: F401

__all__ = ["Grid", "gitter"]
