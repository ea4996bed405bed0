"""GB300-native coupled-cluster hot path of C3L (Coupled-Cluster Coupled Lindblad).

Drop-in replacements for the reference's static CCSD solve, EOM-CCSD sigma
action and retarded Green function, computed by hand-written sm_103a CUDA
kernels behind the C ABI declared in ``include/c3l_gb300.h``.
"""

from .spec import ProblemSpec
from .static import (
    ComponentCCSolution,
    ComponentStaticAction,
    ComponentStaticProblem,
    ContinuationStage,
    NewtonKrylovPolicy,
    NewtonKrylovStep,
    component_static_jvp,
    component_static_residual,
    solve_component_ccsd,
    solve_component_ccsd_continuation,
)
from .matsubara import (
    MatsubaraGreen,
    MatsubaraGrid,
    MatsubaraImpuritySolution,
    MatsubaraSelfEnergy,
    PhysicalModel,
    component_matsubara_green,
    impurity_sites,
    matsubara_dyson_green,
    matsubara_grid,
    matsubara_noninteracting_green,
    matsubara_self_energy,
    noninteracting_retarded_green,
    physical_model,
    solve_matsubara,
)
from .s135 import CompiledFullS135Action, FullS135ResponseOperator
from .spectra import (
    MatrixDysonResult,
    MatrixOrderedReconstruction,
    MatrixResolventDiagnostics,
    MatrixSelfEnergyResult,
    MatrixSpectralDiagnostics,
    PhysicalDysonResult,
    auxiliary_self_energy,
    equilibrium_fdt_defect,
    matrix_auxiliary_self_energy,
    matrix_dyson_green,
    matrix_ordered_dyson_reconstruction,
    matrix_resolvent_diagnostics,
    matrix_spectral_diagnostics,
    noninteracting_auxiliary_green,
    particle_hole_spectral_defect,
    physical_dyson_reconstruction,
    spectral_grid_diagnostics,
)
from .response import (
    ComponentEOMContext,
    ComponentEOMProblem,
    ComponentEOMSources,
    ArnoldiProjection,
    ComponentRetardedGreen,
    ComponentRetardedMatrixArnoldiGreen,
    ComponentRetardedMatrixGreen,
    ComponentRetardedMatrixTime,
    ComponentShiftedMatrixArnoldiGreen,
    ComponentShiftedSolution,
    ComponentSigmaOperator,
    EOMCCSDProblem,
    component_eom_context,
    component_eom_sources,
    component_retarded_green,
    component_retarded_matrix_green,
    component_retarded_matrix_green_arnoldi,
    component_retarded_matrix_green_shifts,
    component_retarded_matrix_time,
    component_retarded_time,
    eom_ccsd_problem,
    solve_component_shifted,
)

__all__ = [
    "ProblemSpec", "ComponentCCSolution", "ComponentStaticAction", "ComponentStaticProblem", "NewtonKrylovPolicy",
    "NewtonKrylovStep", "component_static_jvp", "component_static_residual", "solve_component_ccsd",
    "ComponentEOMContext", "ComponentEOMProblem", "ComponentEOMSources", "ComponentRetardedGreen",
    "ComponentShiftedSolution", "ComponentSigmaOperator", "EOMCCSDProblem", "component_eom_context",
    "component_eom_sources", "component_retarded_green", "eom_ccsd_problem", "ArnoldiProjection",
    "ComponentRetardedMatrixArnoldiGreen", "component_retarded_matrix_green_arnoldi", "solve_component_shifted",
    "ComponentRetardedMatrixGreen", "ComponentRetardedMatrixTime", "ComponentShiftedMatrixArnoldiGreen",
    "component_retarded_matrix_green", "component_retarded_matrix_green_shifts", "component_retarded_matrix_time",
    "component_retarded_time", "MatsubaraGreen", "MatsubaraGrid", "component_matsubara_green", "matsubara_grid",
    "ContinuationStage", "solve_component_ccsd_continuation", "MatrixSelfEnergyResult", "MatsubaraImpuritySolution",
    "MatsubaraSelfEnergy", "PhysicalModel", "impurity_sites", "matrix_auxiliary_self_energy", "matsubara_dyson_green",
    "matsubara_noninteracting_green", "matsubara_self_energy", "noninteracting_retarded_green", "physical_model",
    "solve_matsubara", "CompiledFullS135Action", "FullS135ResponseOperator", "MatrixDysonResult",
    "MatrixOrderedReconstruction", "MatrixResolventDiagnostics", "MatrixSpectralDiagnostics", "PhysicalDysonResult",
    "auxiliary_self_energy", "equilibrium_fdt_defect", "matrix_dyson_green", "matrix_ordered_dyson_reconstruction",
    "matrix_resolvent_diagnostics", "matrix_spectral_diagnostics", "noninteracting_auxiliary_green",
    "particle_hole_spectral_defect", "physical_dyson_reconstruction", "spectral_grid_diagnostics",
]
