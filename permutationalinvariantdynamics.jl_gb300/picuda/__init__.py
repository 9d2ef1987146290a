"""picuda: GB300 backend for the Schur-block Liouvillian hot path of PermutationalInvariantDynamics.jl.

The Python layer mirrors the reference's user-facing API (PIBasis, qubit models,
compile(model; backend=:cuda), apply!, solve_dynamics, stationary_state) over the C ABI of
libpicuda.so (include/picuda.h), whose sm_103a kernels do all numerical work.
"""
from ._lib import (PI_FP32, PI_FP64, PiArgumentError, PiBusy, PiDimensionMismatch, PiError, PiNotConverged,
                   load as load_library)
from .backend import (AcceleratorCapability, CompiledPIModel, DynamicsResult, DynamicsStreamResult,
                      DrivePreconditioner, ExpvAlgorithm, GMRESAlgorithm, HarmonicArnoldiAlgorithm, LevelPreconditioner, drive_preconditioner, drive_preconditioner_tables, level_preconditioner, level_preconditioner_tables, SteadyStateResult, accelerator_capability, apply_, apply_adjoint_, apply_element_major_, element_major_tuning, select_element_major_kernel,
                      compile, engine_schedule_info, evolve_, krylov_expv, krylov_expv_batch, krylov_liouvillian_spectrum, harmonic_arnoldi_spectrum, implicitly_restarted_arnoldi_spectrum, liouvillian_spectrum, pi_liouvillian_gap, SpectrumResult, mul, saved_times, solve_dynamics,
                      solve_dynamics_batch, stationary_state, stationary_state_batch, steady_state,
                      set_engine_schedule, stencil_tables, time_evolve)
from .checkpoints import (PI_CHECKPOINT_VERSION, PIStateCheckpoint, checkpoint_state, load_checkpoint,
                          save_checkpoint)
from .scans import (CompiledPIModelFamily, ParameterScanPlan, ParameterScanPoint, ParameterScanResult,
                    compile_family, parameter_scan, specialize)
from .serving import Completion, Server
from .core import (CollectiveHamiltonian, CollectiveJump, LocalHamiltonian, LocalJump, Models, PIBasis,
                   PIModel, PIOperator, PIState, Term, collective_operator, collective_spin,
                   computational_product_state, expectation, iid_pure_state, qubit_ensemble_model,
                   spin_matrices)

__all__ = [n for n in dir() if not n.startswith("_")]
