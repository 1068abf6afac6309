// Checker for the input-side operations, linked against the reference's own objects by
// oracle/build_ref.sh (test infrastructure: used to generate tests/golden/io.json).
//   qmiv_ref_io color <space 0..3> <to_ycbcr 0|1> <bitdepth> <w> <h> <in.raw> <out.raw>
//     three uint16 planes in, three out: xColorSpace::ConvertRGB2YCbCr / ConvertYCbCr2RGB (the
//     dispatched form the application calls, xAppQMIV.cpp:778-814) -- exits 2 if the portable
//     xColorSpaceSTD::*_I32 result differs from it
//   qmiv_ref_io range <bitdepth> <w> <h> <in.raw> <out.raw>
//     one uint16 plane: prints {"in_range": 0|1} (xPixelOps::CheckIfInRange) and writes the
//     plane after xPixelOps::ClipToRange
#include "xColorSpace.h"
#include "xPixelOps.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

using namespace PMBB_NAMESPACE;

static bool read_all(const char* path, std::vector<uint16>& v)
{
  FILE* f = std::fopen(path, "rb");
  if(!f) return false;
  const size_t n = std::fread(v.data(), sizeof(uint16), v.size(), f);
  std::fclose(f);
  return n == v.size();
}

static bool write_all(const char* path, const std::vector<uint16>& v)
{
  FILE* f = std::fopen(path, "wb");
  if(!f) return false;
  const size_t n = std::fwrite(v.data(), sizeof(uint16), v.size(), f);
  std::fclose(f);
  return n == v.size();
}

int main(int argc, char** argv)
{
  if(argc >= 9 && !std::strcmp(argv[1], "color"))
  {
    const int space = std::atoi(argv[2]), to = std::atoi(argv[3]), bd = std::atoi(argv[4]);
    const int w = std::atoi(argv[5]), h = std::atoi(argv[6]);
    const size_t a = (size_t)w * h;
    std::vector<uint16> in(3 * a), out(3 * a), std_out(3 * a);
    if(!read_all(argv[7], in)) return 1;
    const eClrSpcLC cs = (eClrSpcLC)space;
    if(to)
    {
      xColorSpace::ConvertRGB2YCbCr(out.data(), out.data() + a, out.data() + 2 * a, in.data(), in.data() + a, in.data() + 2 * a, w, w, w, h, bd, cs);
      xColorSpaceSTD::ConvertRGB2YCbCr_I32(std_out.data(), std_out.data() + a, std_out.data() + 2 * a, in.data(), in.data() + a, in.data() + 2 * a, w, w, w, h, bd, cs);
    }
    else
    {
      xColorSpace::ConvertYCbCr2RGB(out.data(), out.data() + a, out.data() + 2 * a, in.data(), in.data() + a, in.data() + 2 * a, w, w, w, h, bd, cs);
      xColorSpaceSTD::ConvertYCbCr2RGB_I32(std_out.data(), std_out.data() + a, std_out.data() + 2 * a, in.data(), in.data() + a, in.data() + 2 * a, w, w, w, h, bd, cs);
    }
    if(!write_all(argv[8], out)) return 1;
    return out == std_out ? 0 : 2;
  }
  if(argc >= 7 && !std::strcmp(argv[1], "range"))
  {
    const int bd = std::atoi(argv[2]), w = std::atoi(argv[3]), h = std::atoi(argv[4]);
    std::vector<uint16> p((size_t)w * h);
    if(!read_all(argv[5], p)) return 1;
    const bool ok = xPixelOps::CheckIfInRange(p.data(), w, w, h, bd);
    xPixelOps::ClipToRange(p.data(), w, w, h, bd);
    std::printf("{\"in_range\": %d}\n", ok ? 1 : 0);
    return write_all(argv[6], p) ? 0 : 1;
  }
  std::fprintf(stderr, "usage: qmiv_ref_io color|range ...\n");
  return 2;
}
