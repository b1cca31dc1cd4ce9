// ibl_hdr.cu -- Radiance RGBE (.hdr) reader and writer for the bake cache
// (host code only).
//
// The reference persists every baked image as a .hdr file and reloads it
// (Src/ImageBasedLighting.cpp:58-102 saveHdriImage, :429-446 cache check,
// :483-568 reload; Src/Utilities.cpp:216-255 loadHdri/saveHdri via the
// un-vendored stb_image / stb_image_write submodule).  This is a restatement
// of the published format (G. Ward, "Real Pixels", Graphics Gems II, 1991,
// and the Radiance file-format notes):
//  * header: "#?RADIANCE" (or "#?RGBE"), variable lines, a blank line, then
//    the resolution string "-Y <h> +X <w>" (top row first);
//  * pixel = R, G, B mantissas + shared exponent E;
//    encode: v = max(r, g, b), v < 1e-32 -> 0, else v = m * 2^e (frexp,
//    m in [0.5, 1)), mantissa = (int)(c * m * 256 / v), E = e + 128;
//    decode: E == 0 -> 0, else c = mantissa * 2^(E - 136);
//  * new-style run-length scanlines for 8 <= w < 32768: marker 2, 2, w>>8,
//    w&255, then each of the four byte planes as runs (count > 128: one byte
//    repeated count - 128 times) or literals (count <= 128).
// Flat (non-RLE) scanlines are read too.  Images are RGBA32F with alpha 1,
// row 0 = the first scanline.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "althea_ibl.h"
#include "ibl_internal.h"

namespace {

void to_rgbe(const float* c, unsigned char* out) {
  float v = c[0];
  if (c[1] > v) v = c[1];
  if (c[2] > v) v = c[2];
  if (!(v >= 1e-32f)) {  // also NaN
    out[0] = out[1] = out[2] = out[3] = 0;
    return;
  }
  int e;
  float m = std::frexp(v, &e);
  float scale = m * 256.0f / v;
  for (int k = 0; k < 3; ++k) {
    float x = c[k] > 0.0f ? c[k] * scale : 0.0f;
    int q = (int)x;
    out[k] = (unsigned char)(q > 255 ? 255 : q);
  }
  int E = e + 128;
  out[3] = (unsigned char)(E < 0 ? 0 : (E > 255 ? 255 : E));
}

void from_rgbe(const unsigned char* in, float* c) {
  if (in[3] == 0) {
    c[0] = c[1] = c[2] = 0.0f;
  } else {
    float f = std::ldexp(1.0f, (int)in[3] - 136);
    c[0] = in[0] * f;
    c[1] = in[1] * f;
    c[2] = in[2] * f;
  }
  c[3] = 1.0f;
}

// One header line without its terminator; "\r\n" endings (files written in
// text mode on Windows) read like "\n" ones.
bool read_line(FILE* f, std::string& line) {
  line.clear();
  int ch;
  while ((ch = fgetc(f)) != EOF) {
    if (ch == '\n') {
      if (!line.empty() && line.back() == '\r') line.pop_back();
      return true;
    }
    line.push_back((char)ch);
    if (line.size() > 4096) return false;
  }
  return !line.empty();
}

// One RLE scanline (after its 4-byte marker) into rgbe[w*4].
bool read_rle_planes(FILE* f, int w, unsigned char* rgbe) {
  for (int p = 0; p < 4; ++p) {
    int x = 0;
    while (x < w) {
      int count = fgetc(f);
      if (count == EOF) return false;
      if (count > 128) {
        count -= 128;
        int v = fgetc(f);
        if (v == EOF || x + count > w) return false;
        for (int k = 0; k < count; ++k) rgbe[4 * (x + k) + p] = (unsigned char)v;
        x += count;
      } else {
        if (count == 0 || x + count > w) return false;
        for (int k = 0; k < count; ++k) {
          int v = fgetc(f);
          if (v == EOF) return false;
          rgbe[4 * (x + k) + p] = (unsigned char)v;
        }
        x += count;
      }
    }
  }
  return true;
}

void write_rle_plane(std::vector<unsigned char>& out, const unsigned char* rgbe, int w, int p) {
  int x = 0;
  while (x < w) {
    // find the next run of >= 4 equal bytes
    int run_start = x, run_len = 0;
    while (run_start < w) {
      run_len = 1;
      while (run_start + run_len < w && run_len < 127 &&
             rgbe[4 * (run_start + run_len) + p] == rgbe[4 * run_start + p])
        ++run_len;
      if (run_len >= 4) break;
      run_start += run_len;
    }
    if (run_start >= w) run_len = 0;
    // literals before the run
    while (x < run_start) {
      int n = run_start - x;
      if (n > 128) n = 128;
      out.push_back((unsigned char)n);
      for (int k = 0; k < n; ++k) out.push_back(rgbe[4 * (x + k) + p]);
      x += n;
    }
    if (run_len >= 4) {
      out.push_back((unsigned char)(128 + run_len));
      out.push_back(rgbe[4 * run_start + p]);
      x = run_start + run_len;
    }
  }
}

}  // namespace

extern "C" int althea_ibl_hdr_read(const char* path, float** rgba_out, int* width, int* height) {
  if (!path || !rgba_out || !width || !height)
    return ibl::set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "null argument");
  *rgba_out = nullptr;
  FILE* f = fopen(path, "rb");
  if (!f) return ibl::set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "cannot open %s", path);
  std::string line;
  bool ok = read_line(f, line) && (line.rfind("#?RADIANCE", 0) == 0 || line.rfind("#?RGBE", 0) == 0);
  bool rgbe = true;
  while (ok && read_line(f, line) && !line.empty()) {
    if (line.rfind("FORMAT=", 0) == 0 && line != "FORMAT=32-bit_rle_rgbe") rgbe = false;
  }
  int w = 0, h = 0;
  char ys[3] = {0}, xs[3] = {0};
  if (ok && rgbe && read_line(f, line) &&
      sscanf(line.c_str(), "%2s %d %2s %d", ys, &h, xs, &w) == 4 && strcmp(ys, "-Y") == 0 &&
      strcmp(xs, "+X") == 0 && w > 0 && h > 0 && w <= 65536 && h <= 65536) {
    std::vector<unsigned char> scan((size_t)w * 4);
    float* img = static_cast<float*>(malloc(sizeof(float) * 4 * (size_t)w * h));
    if (!img) {
      fclose(f);
      return ibl::set_error(ALTHEA_IBL_ERR_OUT_OF_MEMORY, "hdr image");
    }
    for (int y = 0; y < h && ok; ++y) {
      unsigned char head[4];
      if (fread(head, 1, 4, f) != 4) {
        ok = false;
        break;
      }
      if (w >= 8 && w < 32768 && head[0] == 2 && head[1] == 2 && ((head[2] << 8) | head[3]) == w) {
        ok = read_rle_planes(f, w, scan.data());
      } else {  // flat pixels: the 4 bytes just read are the first pixel
        memcpy(scan.data(), head, 4);
        ok = fread(scan.data() + 4, 1, (size_t)(w - 1) * 4, f) == (size_t)(w - 1) * 4;
      }
      for (int x = 0; x < w && ok; ++x) from_rgbe(&scan[4 * x], img + 4 * ((size_t)y * w + x));
    }
    fclose(f);
    if (!ok) {
      free(img);
      return ibl::set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "%s: truncated or corrupt pixels",
                            path);
    }
    *rgba_out = img;
    *width = w;
    *height = h;
    return ALTHEA_IBL_OK;
  }
  fclose(f);
  return ibl::set_error(ALTHEA_IBL_ERR_UNSUPPORTED, "%s: not a 32-bit_rle_rgbe Radiance file",
                        path);
}

extern "C" void althea_ibl_hdr_free(float* p) { free(p); }

extern "C" int althea_ibl_hdr_write(const char* path, const float* rgba, int w, int h) {
  if (!path || !rgba || w < 1 || h < 1 || w > 65536 || h > 65536)
    return ibl::set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "hdr write arguments");
  std::vector<unsigned char> out;
  char head[128];
  int n = snprintf(head, sizeof(head), "#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y %d +X %d\n", h, w);
  out.insert(out.end(), head, head + n);
  std::vector<unsigned char> scan((size_t)w * 4);
  for (int y = 0; y < h; ++y) {
    for (int x = 0; x < w; ++x) to_rgbe(rgba + 4 * ((size_t)y * w + x), &scan[4 * x]);
    if (w >= 8 && w < 32768) {
      out.push_back(2);
      out.push_back(2);
      out.push_back((unsigned char)(w >> 8));
      out.push_back((unsigned char)(w & 255));
      for (int p = 0; p < 4; ++p) write_rle_plane(out, scan.data(), w, p);
    } else {
      out.insert(out.end(), scan.begin(), scan.end());
    }
  }
  FILE* f = fopen(path, "wb");
  if (!f) return ibl::set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "cannot create %s", path);
  bool ok = fwrite(out.data(), 1, out.size(), f) == out.size();
  ok = (fclose(f) == 0) && ok;
  return ok ? ALTHEA_IBL_OK : ibl::set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "write %s", path);
}
