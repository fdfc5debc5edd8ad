"""Mirror of the reference's solver object on top of the C ABI.

The reference drives its solver through `struct ImmerseFlow`
(src/header/globalVariables.cuh:70-88) from `main` (src/main.cu:75-102):

    readInputFile("../inputs/inputs.txt", Solver);
    Solver.CUDAQuery(); Solver.allocation(); Solver.readGridData();
    Solver.initializeData();
    for (t = 0; t < tmax; t++) Solver.ADsolver();
    Solver.freeAllocation();

`ImmerseFlow` below keeps those names and their order of use, and their
meaning: readInputFile parses the keyword grammar, readGridData reads
xgrid/ygrid files, initializeData sets the initial field and iBlank (and
writes final_results.dat when results_dir is set), ADsolver advances one
time step, PPESolver runs the reference's Jacobi Laplace solve, and
freeAllocation writes uc.dat.  Where the reference calls exit(1) on a file
or CUDA error, these methods raise IFXError.
"""
import os

import numpy as np

from . import _capi as capi


class ImmerseFlow:
    def __init__(self, results_dir=None):
        from . import default_config

        self.Input = default_config()
        self.results_dir = results_dir
        self._inputs_dir = "."
        self._xf = None
        self._yf = None
        self._solver = None

    # readInputFile, src/main.cu:10-59
    def readInputFile(self, filename):
        from . import config_read

        self.Input = config_read(filename)
        self._inputs_dir = os.path.dirname(os.path.abspath(filename))

    # CUDAQuery, src/include/preSim.cu:187-199 -- launch geometry is internal here
    def CUDAQuery(self):
        from . import lib

        return lib().ifx_version().decode()

    # allocation, src/include/preSim.cu:147-162 -- done by initializeData
    def allocation(self):
        return None

    # readGridData, src/include/preSim.cu:242-372 (grid files only; centres and
    # widths are built on creation)
    def readGridData(self, xgrid=None, ygrid=None):
        from . import grid_read

        xg = xgrid or self.Input.xgrid.decode()
        yg = ygrid or self.Input.ygrid.decode()
        self._xf = grid_read(xg, self.Input.nx + 1)
        self._yf = grid_read(yg, self.Input.ny + 1)

    def set_grid(self, xf, yf):
        self._xf = np.ascontiguousarray(xf, np.float64)
        self._yf = np.ascontiguousarray(yf, np.float64)

    # initializeData, src/include/preSim.cu:201-240
    def initializeData(self):
        from . import Solver

        if self._xf is None:
            self.readGridData()
        self._solver = Solver.create(self.Input, self._xf, self._yf)
        if self.results_dir:
            self._save(capi.FIELD_IBLANK, "final_results.dat")

    # ADsolver, src/include/ADSolver.cu:268-395 (one time step; the reference
    # also writes uc.dat and vc.dat after every step, src/include/ADSolver.cu:378-379)
    def ADsolver(self):
        self._solver.step(1)
        if self.results_dir:
            self._save(capi.FIELD_U, "uc.dat")
            self._save(capi.FIELD_V, "vc.dat")

    # PPESolver, src/include/PPESolver.cu:137-205
    def PPESolver(self):
        it = self._solver.ppe_reference()
        if self.results_dir:
            self._save(capi.FIELD_P, "p.dat")
        return it

    # freeAllocation, src/include/preSim.cu:164-179
    def freeAllocation(self):
        if self._solver is None:
            return
        if self.results_dir:
            self._save(capi.FIELD_U, "uc.dat")
        self._solver.close()
        self._solver = None

    @property
    def solver(self):
        return self._solver

    def _save(self, field, name):
        from . import write_tecplot

        s = self._solver
        q = s.get(field)
        write_tecplot(os.path.join(self.results_dir, name), s.get(capi.FIELD_XC), s.get(capi.FIELD_YC), q)


def main(inputs="../inputs/inputs.txt", results="../results"):
    """The reference's main(): run tmax steps from inputs.txt, write results."""
    f = ImmerseFlow(results_dir=results)
    f.readInputFile(inputs)
    f.CUDAQuery()
    f.allocation()
    f.readGridData()
    f.initializeData()
    t = 0
    while t < f.Input.tmax:
        f.ADsolver()
        t += 1
    f.freeAllocation()
