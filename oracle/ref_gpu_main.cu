// ref_gpu_main.cu -- assembles the reference program's GPU build.
// TEST INFRASTRUCTURE ONLY (built by oracle/build_ref.py, gpu_build(), into
// oracle/_ref/): the reference's own GPU path on this GPU, a baseline for
// `bench.py --impl reference-shim`, never part of the library.
//
// Order: the shim (geometry, texture references on texture objects), the
// reference's CPU routines, its kernels and host wrappers, then
// osem3d()/main(), each extracted verbatim from the reference sources.
#include "ref_gpu_shim.cuh"

#include "ref_cpu.inc"
#include "ref_kernels.inc"
#include "ref_gpu_host.inc"
#include "ref_driver.inc"
