// ref_main.cpp -- assembles the host-emulated reference program.
// TEST INFRASTRUCTURE ONLY (built by oracle/build_ref.py into oracle/_ref/).
//
// Order: shim, the reference's CPU file (compiled where it lies, -I of the
// reference tree), the kernels extracted from GFIRST_GPU_Kernels.cu, the
// host launch wrappers below (same grid/block shapes as the reference's),
// then osem3d()/main() extracted from GFIRST.cu.
#include "ref_shim.h"

#include "GFIRST_CPU_Kernels.cpp"

#include "ref_kernels.inc"

// Host wrappers, launch shapes of GFIRST_GPU_Kernels.cu.
void FORWPROJ(float* d_PROJ, int itheta, int idz, int iTOF) {
  gfref_launch(dim3(NZS), dim3(NRAD), [=] { FORWPROJ_K(d_PROJ, itheta, idz, iTOF); });
}
void BACKWPROJ(float* d_NUMER, float* d_DENOM, int itheta, int idz, int iTOF) {
  gfref_launch(dim3(RES, NZS), dim3(RES, 1), [=] { BACKWPROJ_K(d_NUMER, d_DENOM, itheta, idz, iTOF); });
}
void dividirVxVGPU(float* d_vA, float* d_vB, int els, float* d_vR) {
  gfref_launch(dim3(RES, NZS), dim3(RES, 1), [=] { divVxVGPU(d_vA, d_vB, els, d_vR); });
}
void CleanMemory(float* mem, int size) {
  int bloques = (int)ceil(size / (float)BSX);
  gfref_launch(dim3(bloques, 1), dim3(BSX, 1), [=] { CleanMemoryK(mem, size); });
}
void convolutionXY(float* d_volume, float* d_tempVolume) {
  gfref_launch_sync(dim3(NZS, 1), dim3(RES, 1), [=] { convolutionXY_GPU(d_volume, d_tempVolume); });
}
void jointbilateralfilter3D(float* input, float* reference, float max_ref, int r, float sigma3D, float sigmaI,
                            float* output) {
  gfref_launch(dim3(RES, NZS), dim3(RES, 1),
               [=] { jointbilateralfilter3D_K(input, reference, max_ref, r, sigma3D, sigmaI, output); });
}
static void gfref_fill(texture<float, 3>& t, const float* h) {
  memcpy(t.data.data(), h, sizeof(float) * t.data.size());
}
void UpdateImage(float* h_imagen) { gfref_fill(imgEstTex, h_imagen); }
void actualizarCorr(float* h_imagen) { gfref_fill(CorrTex, h_imagen); }
void actualizarCalib(float* h_imagen) { gfref_fill(CalibTex, h_imagen); }
void crearTexturas() {
  imgEstTex.w = RES; imgEstTex.h = RES; imgEstTex.d = NZS;
  imgEstTex.data.assign((size_t)RES * RES * NZS, 0.f);
  CorrTex.w = NRAD; CorrTex.h = NZS; CorrTex.d = 1;
  CorrTex.data.assign((size_t)NRAD * NZS, 0.f);
  CalibTex.w = NRAD; CalibTex.h = NZS; CalibTex.d = 1;
  CalibTex.data.assign((size_t)NRAD * NZS, 0.f);
}

#define main gfref_main
#include "ref_driver.inc"
#undef main

int main(int argc, char** argv) { return gfref_main(argc, argv); }
