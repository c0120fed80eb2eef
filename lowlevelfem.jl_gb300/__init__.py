"""lowlevelfem.jl_gb300 — GB300-native operator assembly and iterative solve
behind LowLevelFEM.jl's API (stiffnessMatrix, massMatrix,
heatConductionMatrix, the Total Lagrangian trio, solveDisplacement,
solveTemperature, solveField).

The directory name is not a Python identifier; import it through
``__graft_entry__.load_package()`` (or importlib), which registers it as the
module ``llfem_gb300``.
"""
from . import _lib
from ._lib import LLFError, Context, default_context
from .mesh import (Mesh, Group, structured_rect_mesh, structured_box_mesh, read_msh,
                   current_mesh, set_current, node_lattice, concat_meshes, LINE, TRI, QUAD, TET, HEX)
from .api import (Material, material, elastic_constants, Problem, Field, SystemMatrix, VectorField,
                  ScalarField, TensorField, BoundaryCondition, LoadCondition, displacementConstraint,
                  temperatureConstraint, load, heatFlux, elasticSupport, heatConvection, constrainedDoFs,
                  allDoFs, freeDoFs, applyBoundaryConditions_, loadVector, stiffnessMatrix, autotune, massMatrix,
                  heatConductionMatrix, heatCapacityMatrix, elasticSupportMatrix, heatConvectionMatrix,
                  heatConvectionVector, applyElasticSupport_, applyHeatConvection_, externalTangentFollower,
                  elementsToNodes, isElementwise, solveDisplacement,
                  solveTemperature, solveField, solveFieldBatched, FDM, grad,
                  deformationGradient, materialTangentMatrix, initialStressMatrix, tangentMatrix, solveDeformation,
                  internalForceVector)

from .dsl import OpApplied, BilinearTerm, Grad, SymGrad, Id, integrate, build_csc_pattern

__version__ = "0.1.0"
