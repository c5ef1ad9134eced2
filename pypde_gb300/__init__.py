"""pypde_gb300 -- PyPDE's ADER-WENO time step on one GB300 GPU.

Drop-in for ``pypde.pde_solver`` / ``pypde.weno_solver`` (haranjackson/PyPDE
pypde/__init__.py): same arguments, same result layout, every stage of the
step run by hand-written sm_103a kernels in libpypde_gb300.so.
"""
from .solvers import ader_solver, pde_solver, pde_solver_batch, weno_solver  # noqa: F401
from . import systems  # noqa: F401
