// gf_io.cpp -- the reference's raw file formats (host only).
#include <cstdio>
#include <cstring>
#include <vector>

#include "gf_internal.h"

using namespace gf;

static long file_size(FILE* f) {
  if (fseek(f, 0L, SEEK_END) != 0) return -1;
  long n = ftell(f);
  fseek(f, 0L, SEEK_SET);
  return n;
}

extern "C" {

// ReadSinogram_Type, GFIRST_CPU_Kernels.cpp:104-142.  The reference reads all
// of the file into a 2*NDATA buffer without a bound; words past 2*NDATA are
// ignored here.
gf_status gf_read_sinogram(const char* path, int64_t ndata, float* h_out) {
  if (!path || !h_out || ndata <= 0) return set_error(GF_ERR_ARG, "bad argument");
  const int64_t n = 2 * ndata;
  memset(h_out, 0, (size_t)n * sizeof(float));
  FILE* f = fopen(path, "rb");
  if (!f) return set_error(GF_ERR_IO, std::string("Sinogram Not Found: ") + path);
  long bytes = file_size(f);
  int64_t words = bytes > 0 ? bytes / 4 : 0;
  int64_t m = words < n ? words : n;
  std::vector<int32_t> ints((size_t)m);
  size_t got = m ? fread(ints.data(), 4, (size_t)m, f) : 0;
  fclose(f);
  if ((int64_t)got != m) return set_error(GF_ERR_IO, std::string("short read: ") + path);
  float mx = 0.f;
  for (int64_t i = 0; i < m; i++) {
    h_out[i] = (float)ints[i];
    if (h_out[i] > mx) mx = h_out[i];
  }
  if (mx > 1.0e6) memcpy(h_out, ints.data(), (size_t)m * 4);  // float32 file
  return GF_OK;
}

// ReadImage, GFIRST_CPU_Kernels.cpp:58-66 (a short file leaves zeros).
gf_status gf_read_image(const char* path, int64_t nvox, float* h_out) {
  if (!path || !h_out || nvox <= 0) return set_error(GF_ERR_ARG, "bad argument");
  memset(h_out, 0, (size_t)nvox * sizeof(float));
  FILE* f = fopen(path, "rb");
  if (!f) return set_error(GF_ERR_IO, std::string("Image Not Found: ") + path);
  size_t got = fread(h_out, sizeof(float), (size_t)nvox, f);
  (void)got;
  fclose(f);
  return GF_OK;
}

// VLOR records as GFIRST.cu:232-240 reads them: int32 pairs; its
// `while (!feof)` loop runs the body once more after the last full record
// with what the failed fread left in the buffer (the last record, or, when
// 4-7 bytes remain, the new first word with the old second word).
gf_status gf_read_vlor(const char* path, int32_t* h_events, int64_t* nevents) {
  if (!path || !nevents) return set_error(GF_ERR_ARG, "bad argument");
  FILE* f = fopen(path, "rb");
  if (!f) return set_error(GF_ERR_IO, std::string("VLOR file Not Found: ") + path);
  long bytes = file_size(f);
  int64_t nfull = bytes > 0 ? bytes / 8 : 0;
  int64_t total = nfull > 0 ? nfull + 1 : 0;
  if (!h_events) {
    fclose(f);
    *nevents = total;
    return GF_OK;
  }
  if (*nevents < total) {
    fclose(f);
    *nevents = total;
    return set_error(GF_ERR_ARG, "event buffer too small");
  }
  size_t got = nfull ? fread(h_events, 8, (size_t)nfull, f) : 0;
  if ((int64_t)got != nfull) {
    fclose(f);
    return set_error(GF_ERR_IO, std::string("short read: ") + path);
  }
  if (nfull > 0) {
    int32_t last[2] = {h_events[2 * nfull - 2], h_events[2 * nfull - 1]};
    if (bytes % 8 >= 4) {
      int32_t w;
      if (fread(&w, 4, 1, f) == 1) last[0] = w;
    }
    h_events[2 * nfull] = last[0];
    h_events[2 * nfull + 1] = last[1];
  }
  fclose(f);
  *nevents = total;
  return GF_OK;
}

// VLOR events as two LORs of endpoints each: 48-byte records of 12 float32.
gf_status gf_read_vlor_endpoints(const char* path, float* h_lors, int64_t* nevents) {
  if (!path || !nevents) return set_error(GF_ERR_ARG, "bad argument");
  FILE* f = fopen(path, "rb");
  if (!f) return set_error(GF_ERR_IO, std::string("VLOR file Not Found: ") + path);
  long bytes = file_size(f);
  const int64_t n = bytes > 0 ? bytes / 48 : 0;
  if (!h_lors) {
    fclose(f);
    *nevents = n;
    return GF_OK;
  }
  if (*nevents < n) {
    fclose(f);
    *nevents = n;
    return set_error(GF_ERR_ARG, "event buffer too small");
  }
  size_t got = n ? fread(h_lors, 48, (size_t)n, f) : 0;
  fclose(f);
  if ((int64_t)got != n) return set_error(GF_ERR_IO, std::string("short read: ") + path);
  *nevents = n;
  return GF_OK;
}

// WriteImage, GFIRST_CPU_Kernels.cpp:25-33.
gf_status gf_write_raw(const char* path, const float* h_data, int64_t n) {
  if (!path || (!h_data && n) || n < 0) return set_error(GF_ERR_ARG, "bad argument");
  FILE* f = fopen(path, "wb");
  if (!f) return set_error(GF_ERR_IO, std::string("cannot write ") + path);
  size_t put = n ? fwrite(h_data, sizeof(float), (size_t)n, f) : 0;
  fclose(f);
  if ((int64_t)put != n) return set_error(GF_ERR_IO, std::string("short write: ") + path);
  return GF_OK;
}

}  // extern "C"
