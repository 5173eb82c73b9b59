"""GB300-native SPARC wave-solver hot path: the option-17 time step (linearised displacement
equations about a stratified background with flows, physics2d.f90:943-1094) with its PML, RK
update, records and sensitivity-kernel integral, as hand-written sm_103a CUDA behind a C ABI
(include/sparc_gb300.h, built into _lib/libsparc_gb300.so by _build.py).  There is no CPU
fallback: without the library nothing here computes.

Modules (reference counterpart in parentheses):
  solver          WaveSolver: a batch of 2-D solves on one GPU (STEP, TIMESTEPPING)
  pipeline        FwdAdjKernels: forward, reference-style adjoint and kernel integral of a batch,
                  partial states in HBM or checkpointed (full.py's three sparc runs, PRODUCE_KERNELS)
  discrete_adjoint  exact discrete adjoint of the step: flow and sound-speed gradients
  autograd        torch.autograd wrappers of both adjoints
  fdcheck         central-difference check of the exact gradient
  cli, bin/sparc  the `sparc NN MM` executable contract (driver.f90, READ_PARAMETERS)
  full_batched    full.py's per-source loop as one batched process, same files
  linesearch_batched  linesearch.py's forward runs of all sources and trial models in one batch
  ttadjoint       travel-time adjoint source and misfits (ADJOINT_SOURCE_FILT, MISFIT_ALL)
  gradient, bin/grad.py  gradient post-processing and update directions (grad.py)
  fits, fits_gpu  FITS files and partial-state dumps (all_modules.f90)
  solver3d        3-D forward step (option 16)
  solver_sponge   velocity-pressure-density steps (options 5, 6, 12)
  uneven          batches of solves of different sizes and lengths
  model, config   synthetic backgrounds, sources, params.i parsing
  accuracy        FP32 against FP64 error report
  distributed     sources sharded over ranks, kernel sums
"""
