"""GB300 (sm_103a) backend of Wavey's FDTD wave solver.

  backend    CudaBackend over libwavey_cuda.so: run_fdtd / run_batch / plan /
             run_rooms / build_grid, device-resident plans (autotune,
             transfers, band_params)
  fdtd       grids, taps, source components, signals and transfer functions
             over libwavey_host.so (fdtd.rs)
  materials  materials and admittance fits (impedance_fit.rs, material.rs)
  wave       the wave stage of a solve as batched launches (run.rs:593-662),
             cabinet calibrations (fdtd.rs:890-955), the results.bin
             transfer section
  workloads  the seeded synthetic benchmark scenes
"""
