// gf_cli.cpp -- `gfirst`, the drop-in for the reference's command line
// (GFIRST.cu:577-621).  The number of positional arguments picks the mode
// exactly as there:
//   gfirst image.raw                                  projection -> proj_ref.raw
//   gfirst sino.raw norm.raw                          doubles
//   gfirst sinoD.raw sinoT.raw norm.raw               doubles + triples
//   gfirst sinoD.raw sinoT.raw norm.raw vlor.raw      doubles + triples VLOR
// and the outputs have the reference's names: proj_ref.raw,
// img_GPU_D_ITER%d.raw / img_GPU_T_ITER%d.raw every 20 iterations, and
// SINOG_VLOR.raw.  Options (before or after the files) change what the
// reference fixes at compile time:
//   --geometry res,nzs,nrad,nang,span,nseg,pitch,diam,fov   (default GFIRST.h)
//   --subsets S  --iterations N  --write-every K  --device D
//   --vlor-endpoints   the VLOR file holds two LORs of float32 endpoints per
//                      event (gf_read_vlor_endpoints) instead of int32 bins
//   --storage f32|f16|bf16   element type of the per-subset ratio sinogram
//                            (arithmetic stays FP32; default f32)
//   --image-storage f32|f16|bf16   element type of the reconstructed images
//                                  between sub-iterations (default f32)
//   --tune             pick the projectors' tile shapes by timing first
//   --bp-form view|voxel   the back projector's axial interpolation for the
//                          doubles image (gf_set_bp_form; default view)
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gfirst.h"

static int usage() {
  printf("1 Input  --> Projection [Input = 3D Image] \n");
  printf("2 Inputs --> Reconstruction [Input = Sinog_Doubles + Sinog_Normalization]\n");
  printf("3 Inputs --> Reconstruction Doubles & Triples [Input = Sinog_Doubles + Sinog_Triples + Sinog_Normalization] \n");
  printf("4 Inputs --> VLOR reconstruction [Input = Sinog_Doubles + Sinog_Triples + Sinog_Normalization + Vlor_file] \n");
  printf("options: --geometry res,nzs,nrad,nang,span,nseg,pitch,diam,fov --subsets S --iterations N "
         "--write-every K --device D --vlor-endpoints --storage f32|f16|bf16 --image-storage f32|f16|bf16 --tune "
         "--bp-form view|voxel\n");
  return 0;
}

static int die(const char* what, gf_status st) {
  fprintf(stderr, "gfirst: %s failed (%d): %s\n", what, (int)st, gf_last_error());
  return 1;
}

int main(int argc, char** argv) {
  gf_geometry g;
  gf_geometry_reference(&g);
  int nsub = 1, niter = -1, every = 20, device = 0;
  bool vlor_endpoints = false, tune = false;
  int bp_form = GF_BP_PER_VIEW;
  int storage = GF_STORE_F32, image_storage = GF_STORE_F32;
  std::vector<std::string> files;
  for (int i = 1; i < argc; i++) {
    std::string a = argv[i];
    auto val = [&](const char* name) -> const char* {
      if (i + 1 >= argc) {
        fprintf(stderr, "gfirst: %s needs a value\n", name);
        exit(2);
      }
      return argv[++i];
    };
    if (a == "--geometry") {
      const char* v = val("--geometry");
      if (sscanf(v, "%d,%d,%d,%d,%d,%d,%f,%f,%f", &g.res, &g.nzs, &g.nrad, &g.nang, &g.span, &g.nseg, &g.pitch_mm,
                 &g.diam_det_mm, &g.fov_mm) != 9) {
        fprintf(stderr, "gfirst: --geometry wants 9 comma-separated values\n");
        return 2;
      }
    } else if (a == "--subsets") {
      nsub = atoi(val("--subsets"));
    } else if (a == "--iterations") {
      niter = atoi(val("--iterations"));
    } else if (a == "--write-every") {
      every = atoi(val("--write-every"));
    } else if (a == "--device") {
      device = atoi(val("--device"));
    } else if (a == "--vlor-endpoints") {
      vlor_endpoints = true;
    } else if (a == "--tune") {
      tune = true;
    } else if (a == "--bp-form") {
      const std::string v = val("--bp-form");
      if (v == "view") bp_form = GF_BP_PER_VIEW;
      else if (v == "voxel") bp_form = GF_BP_PER_VOXEL;
      else {
        fprintf(stderr, "gfirst: --bp-form wants view or voxel\n");
        return 2;
      }
    } else if (a == "--storage" || a == "--image-storage") {
      const std::string v = val(a.c_str());
      int* dst = a == "--storage" ? &storage : &image_storage;
      if (v == "f32") *dst = GF_STORE_F32;
      else if (v == "f16") *dst = GF_STORE_F16;
      else if (v == "bf16") *dst = GF_STORE_BF16;
      else {
        fprintf(stderr, "gfirst: %s wants f32, f16 or bf16\n", a.c_str());
        return 2;
      }
    } else if (a == "-h" || a == "--help") {
      return usage();
    } else {
      files.push_back(a);
    }
  }
  if (files.empty() || files.size() > 4) return usage();
  const int mode = (int)files.size() - 1;
  int64_t planes, ndata, nvox;
  gf_status st = gf_geometry_sizes(&g, &planes, &ndata, &nvox);
  if (st != GF_OK) return die("geometry", st);
  gf_ctx* ctx = nullptr;
  if ((st = gf_create(&g, nsub, device, &ctx)) != GF_OK) return die("gf_create", st);
  if ((st = gf_set_bp_form(ctx, bp_form)) != GF_OK) return die("gf_set_bp_form", st);
  gf_recon_params p;
  gf_recon_defaults(mode, &p);
  if (niter >= 0) p.niter = niter;
  p.storage = storage;
  p.image_storage = image_storage;
  if (tune) {
    int32_t R, chunk, warps;
    if ((st = gf_tune(ctx, &R, &chunk, &warps)) != GF_OK) return die("gf_tune", st);
    printf("Tile shapes: R %d, %d steps per chunk, %d back-projector warps\n", R, chunk, warps);
  }
  gf_recon* r = nullptr;
  if ((st = gf_recon_create(ctx, &p, &r)) != GF_OK) return die("gf_recon_create", st);
  printf("Starting............ \n");
  std::vector<float> image, dsino, tsino, norm;
  std::vector<int32_t> ev;
  int64_t nev = 0;
  if (mode == 0) {
    printf("Reading Input Image for Projection ... \n");
    image.resize(nvox);
    if ((st = gf_read_image(files[0].c_str(), nvox, image.data())) != GF_OK) return die("read image", st);
  } else {
    const char* normf = files[mode == 1 ? 1 : 2].c_str();
    norm.resize(2 * ndata);
    if (gf_read_sinogram(normf, ndata, norm.data()) != GF_OK) printf("Sinogram Not Found!\n");
    printf("Normalization Sinogram loaded \n");
    dsino.resize(2 * ndata);
    if (gf_read_sinogram(files[0].c_str(), ndata, dsino.data()) != GF_OK) printf("Sinogram Not Found!\n");
    if (mode >= 2) {
      tsino.resize(2 * ndata);
      if (gf_read_sinogram(files[1].c_str(), ndata, tsino.data()) != GF_OK) printf("Sinogram Not Found!\n");
    }
    if (mode == 3 && !vlor_endpoints) {
      printf("Reading VLOR file \n");
      if ((st = gf_read_vlor(files[3].c_str(), nullptr, &nev)) != GF_OK) return die("read VLOR", st);
      ev.resize(2 * (size_t)nev + 2);
      if ((st = gf_read_vlor(files[3].c_str(), ev.data(), &nev)) != GF_OK) return die("read VLOR", st);
    } else if (mode == 3) {
      printf("Reading VLOR file (LOR endpoints) \n");
      if ((st = gf_read_vlor_endpoints(files[3].c_str(), nullptr, &nev)) != GF_OK) return die("read VLOR", st);
      std::vector<float> lors(12 * (size_t)nev + 12);
      if ((st = gf_read_vlor_endpoints(files[3].c_str(), lors.data(), &nev)) != GF_OK) return die("read VLOR", st);
      ev.resize(2 * (size_t)nev + 2);
      void *dl = nullptr, *de = nullptr;
      if ((st = gf_device_alloc(ctx, lors.size() * sizeof(float), &dl)) != GF_OK) return die("alloc", st);
      if ((st = gf_device_alloc(ctx, ev.size() * sizeof(int32_t), &de)) != GF_OK) return die("alloc", st);
      if ((st = gf_copy_to_device(ctx, dl, lors.data(), lors.size() * sizeof(float))) != GF_OK) return die("copy", st);
      if ((st = gf_vlor_from_endpoints(ctx, static_cast<const float*>(dl), nev, static_cast<int32_t*>(de))) != GF_OK)
        return die("VLOR endpoints", st);
      if ((st = gf_copy_to_host(ctx, ev.data(), de, ev.size() * sizeof(int32_t))) != GF_OK) return die("copy", st);
      gf_device_free(ctx, dl);
      gf_device_free(ctx, de);
    }
    double sumd = 0, sumdbg = 0;
    for (int64_t i = 0; i < ndata; i++) {
      sumd += dsino[i];
      sumdbg += dsino[ndata + i];
    }
    printf("  Doubles Coincidences: Prompts= %.1f Million, Background= %.1f Million\n", sumd / 1.0e6, sumdbg / 1.0e6);
  }
  auto t0 = std::chrono::steady_clock::now();
  st = gf_recon_load(r, image.empty() ? nullptr : image.data(), dsino.empty() ? nullptr : dsino.data(),
                     tsino.empty() ? nullptr : tsino.data(), norm.empty() ? nullptr : norm.data(),
                     ev.empty() ? nullptr : ev.data(), nev);
  if (st != GF_OK) return die("gf_recon_load", st);
  {
    std::vector<float> pr(ndata);
    if ((st = gf_recon_get_proj_ref(r, pr.data())) != GF_OK) return die("get proj_ref", st);
    if ((st = gf_write_raw("proj_ref.raw", pr.data(), ndata)) != GF_OK) return die("write proj_ref.raw", st);
  }
  if (mode == 0) {
    printf("Finish After Projection \n");
  } else {
    std::vector<float> out(nvox);
    for (int it = 1; it <= p.niter; it++) {
      printf("ITER= %d  \n", it);
      if ((st = gf_recon_iterate(r, 1)) != GF_OK) return die("iterate", st);
      if (every > 0 && it % every == 0) {
        char name[256];
        snprintf(name, sizeof name, "img_GPU_D_ITER%d.raw", it);
        if ((st = gf_recon_get_image(r, 0, 1, out.data())) != GF_OK) return die("get image", st);
        gf_write_raw(name, out.data(), nvox);
        if (mode > 1) {
          snprintf(name, sizeof name, "img_GPU_T_ITER%d.raw", it);
          if ((st = gf_recon_get_image(r, 1, 1, out.data())) != GF_OK) return die("get image", st);
          gf_write_raw(name, out.data(), nvox);
        }
      }
    }
    if (mode == 3 && p.niter > 0) {
      std::vector<float> v(ndata);
      if ((st = gf_recon_get_sinog_vlor(r, v.data())) != GF_OK) return die("get SINOG_VLOR", st);
      gf_write_raw("SINOG_VLOR.raw", v.data(), ndata);
    }
  }
  gf_synchronize(ctx);
  double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  printf("\nTotal Time: %f (s) \n", dt);
  gf_recon_destroy(r);
  gf_destroy(ctx);
  return 0;
}
