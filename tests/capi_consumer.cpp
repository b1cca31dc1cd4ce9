// A C++ caller of the C ABI, built and run by tests/test_capi.py without a
// GPU: it links libalthea_ibl.so the way the engine's precompute code would
// (the reference is C++, Src/ImageBasedLighting.cpp) and exercises the calls
// that need no device -- the reference configuration, chain geometry, the
// precision planner, the RGBE files and the error reporting.  Exit status 0
// means every check held; otherwise the first failed check is printed.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "althea_ibl.h"

#define CHECK(cond)                                                        \
  do {                                                                     \
    if (!(cond)) {                                                         \
      std::fprintf(stderr, "check failed at line %d: %s\n", __LINE__, #cond); \
      return 1;                                                            \
    }                                                                      \
  } while (0)

int main(int argc, char** argv) {
  const std::string dir = argc > 1 ? argv[1] : ".";

  // createResources' settings (Src/ImageBasedLighting.cpp:184-221).
  althea_ibl_config cfg;
  althea_ibl_config_reference(&cfg, 4096, 2048);
  CHECK(cfg.mip_count == 5 && cfg.first_mip_width == 2048 && cfg.samples == 10000);
  CHECK(althea_ibl_chain_levels(4096, 2048) == 13);
  CHECK(althea_ibl_chain_level_offset(4096, 2048, 1) == (size_t)4096 * 2048);

  // The precision planner for a 9-mip chain from 2048x1024 and a 128x64 irradiance.
  althea_ibl_mip_target mips[9];
  for (int m = 0; m < 9; ++m) {
    mips[m].out_dev = nullptr;
    mips[m].width = 2048 >> m;
    mips[m].height = 1024 >> m;
    mips[m].pitch_bytes = (size_t)mips[m].width * 16;
    mips[m].roughness = (float)m / 8.0f;
  }
  int levels[9], irr_level = -9;
  CHECK(althea_ibl_tc_plan(4096, 2048, mips, 9, 128, levels, &irr_level) == ALTHEA_IBL_OK);
  CHECK(levels[0] == -1 && levels[1] == 2 && levels[8] == 1 && irr_level == 1);
  CHECK(althea_ibl_tc_workspace_size(4096, 2048, mips, 9, levels, 128, 64, irr_level) > 0);

  // Errors come back as a status and a message, never as an exception.
  althea_ibl_config bad = cfg;
  bad.mip_count = 0;
  althea_ibl_context* ctx = nullptr;
  CHECK(althea_ibl_create(&bad, &ctx) == ALTHEA_IBL_ERR_INVALID_ARGUMENT && ctx == nullptr);
  CHECK(std::string(althea_ibl_last_error()).find("mip_count") != std::string::npos);

  // An RGBE file written and read back (the bake cache's format).
  const int w = 40, h = 3;
  std::vector<float> img((size_t)w * h * 4);
  for (int i = 0; i < w * h; ++i) {
    img[4 * i + 0] = 0.5f + i;
    img[4 * i + 1] = 1.0f;
    img[4 * i + 2] = i % 7 == 0 ? 1e5f : 0.25f;
    img[4 * i + 3] = 1.0f;
  }
  const std::string path = dir + "/consumer.hdr";
  CHECK(althea_ibl_hdr_write(path.c_str(), img.data(), w, h) == ALTHEA_IBL_OK);
  float* back = nullptr;
  int bw = 0, bh = 0;
  CHECK(althea_ibl_hdr_read(path.c_str(), &back, &bw, &bh) == ALTHEA_IBL_OK);
  CHECK(bw == w && bh == h && back != nullptr);
  for (int i = 0; i < w * h; ++i) {
    const float mx = std::fmax(img[4 * i], std::fmax(img[4 * i + 1], img[4 * i + 2]));
    for (int c = 0; c < 3; ++c) CHECK(std::fabs(back[4 * i + c] - img[4 * i + c]) <= mx / 128);
    CHECK(back[4 * i + 3] == 1.0f);
  }
  althea_ibl_hdr_free(back);
  CHECK(althea_ibl_hdr_read((dir + "/missing.hdr").c_str(), &back, &bw, &bh) ==
        ALTHEA_IBL_ERR_INVALID_ARGUMENT);
  std::printf("consumer ok\n");
  return 0;
}
