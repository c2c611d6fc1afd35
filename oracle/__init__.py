"""The oracle: a CPU restatement of wavey-solver's FDTD path.

TEST INFRASTRUCTURE, NOT PRODUCT CODE.  Only tests/, __graft_entry__.smoke()
and bench.py's CPU-baseline leg load anything from this package; the
product (wavey_gb300) never imports it.

  fdtd_oracle.c  run_cpu / run_cpu_ir in FP64 (fdtd.rs:644-725), and the same
                 loop in FP32 in the reference shader's operation order
                 (fdtd.wgsl:44-119), compiled by build.py into
                 oracle/_build/libwavey_oracle.so
  fp16_oracle.c  the FP32 loop with the fields stored as FP16 times a power of
                 two per z slab and time level (the FP16-storage form of the
                 CUDA path: slab scales, rounding, slab maxima)
  ir_oracle.c    the IR post-processing (analysis.rs:143-325): octave
                 band-pass, onset, Schroeder / Lundeby, ISO 3382-1 parameters
  voxel.py       numpy restatement of FdtdGrid::build_dx (fdtd.rs:289-378)
                 and boundary_slots (fdtd.rs:539-571) for box rooms

Parity pins: the reference stores no golden vectors for this path; the
oracle is pinned by the reference's own known-answer tests
(core/wavey-solver/tests/fdtd.rs), ported in tests/test_oracle_pins.py.
"""
