"""GB300-native (sm_103a) HDG Poisson path of HDiscontinuousGalerkin.jl.

The public names mirror the reference's Julia API (a trailing underscore stands for Julia's
`!`): rectangle_mesh, parse_mesh_triangle, GenericFiniteElement(Dubiner(...)),
ScalarFunctionSpace, VectorFunctionSpace, ScalarTraceFunctionSpace, TrialFunction, Dirichlet,
CellIterator, start_assemble / assemble_ / end_assemble, doassemble, apply_, solve,
get_usigma_, errornorm.  Everything numerical runs in libhdg.so (CUDA, built in-tree)."""
from . import _lib
from ._lib import HDGError, PREC_FP64, PREC_MIXED, PRECOND_AMG, PRECOND_JACOBI
from .batch import Batch, Problem, concat_meshes, problem_offsets
from .serve import Engine
from .vtk import write_vtk
from .lagrange import LagrangeSystem, doassemble_cg, reconstruct_
from .assembler import Assembler, SparseMatrixCSC, assemble_, end_assemble, start_assemble
from .context import Context, default_context
from .fields import MANUFACTURED_F, MANUFACTURED_U, Field
from .mesh import (Cell, PolygonalMesh, TriangleCell, cell_diameter, face_orientation, get_coordinates,
                   get_vertices_matrix, getcells_matrix, getfaceset, getncells, getnfaces, getnnodes,
                   n_faces_per_cell, parse_mesh_triangle, rectangle_mesh)
from .dofhandler import (AssemblerSparsityPattern, DofHandler, celldofs_, create_sparsity_pattern,
                         create_symmetric_sparsity_pattern, dof_range, ndofs, ndofs_per_cell, nvariables)
from .spaces import (ContinuousLagrange, Dubiner, GenericFiniteElement, Legendre, RefTetrahedron, ScalarFunctionSpace,
                     ScalarTraceFunctionSpace, VectorFunctionSpace, get_normal, getdetJdV, getfacedetJdS,
                     getnbasefunctions, getnfacequadpoints, getnlocaldofs, getnquadpoints, reinit_, shape_divergence,
                     shape_gradient, shape_value)
from .system import (CellIterator, Dirichlet, SolveStats, TraceSystem, TrialFunction, apply_, doassemble, errornorm,
                     get_usigma_, nodal_avg, solve, solve_poisson)


def load_library():
    """Build (if needed) and load libhdg.so; raises if that is impossible."""
    return _lib.load()
