// Drives the C++ processors of include/qmiv_gb300.hpp the way xAppQMIV drives the reference's:
//   shim_demo probe                               -> tries to create a processor, prints the status
//   shim_demo W H BD ref.raw tst.raw [erp]        -> all metrics of one 4:2:0 uint16 pair as JSON
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "qmiv_gb300.hpp"

using namespace qmiv_gpu;

static bool read_raw(const char* path, std::vector<uint16_t>& v)
{
  FILE* f = std::fopen(path, "rb");
  if(!f) return false;
  const size_t n = std::fread(v.data(), sizeof(uint16_t), v.size(), f);
  std::fclose(f);
  return n == v.size();
}

int main(int argc, char** argv)
{
  if(argc >= 2 && !std::strcmp(argv[1], "probe"))
  {
    try { xIVPSNR_GPU p; p.create(64, 64); std::printf("{\"status\": 0}\n"); }
    catch(const Error& e) { std::printf("{\"status\": %d}\n", (int)e.status); }
    return 0;
  }
  if(argc < 6) { std::fprintf(stderr, "usage: shim_demo W H BD ref.raw tst.raw [erp]\n"); return 2; }
  const int W = std::atoi(argv[1]), H = std::atoi(argv[2]), BD = std::atoi(argv[3]);
  const bool erp = argc > 6 && !std::strcmp(argv[6], "erp");
  const size_t a = (size_t)W * H, ca = (size_t)(W / 2) * (H / 2);
  std::vector<uint16_t> ref(a + 2 * ca), tst(a + 2 * ca);
  if(!read_raw(argv[4], ref) || !read_raw(argv[5], tst)) { std::fprintf(stderr, "cannot read inputs\n"); return 2; }
  // picture 0 = Tst, picture 1 = Ref, as in the application
  const qmiv_pic P0 = make_pic_planar(tst.data(), tst.data() + a, tst.data() + a + ca, W, W / 2, W, H, BD, QMIV_CF420, false);
  const qmiv_pic P1 = make_pic_planar(ref.data(), ref.data() + a, ref.data() + a + ca, W, W / 2, W, H, BD, QMIV_CF420, false);
  try
  {
    xPSNR_GPU psnr;
    xWSPSNR_GPU wspsnr;
    xIVPSNR_GPU ivpsnr;
    xSSIM_GPU ssim;
    xIVSSIM_GPU ivssim;
    wspsnr.initWS(erp, W, H, BD);
    ivpsnr.initWS(erp, W, H, BD);
    ssim.create(W, H, BD, 0, true);
    const int32V4 gcd = ivpsnr.CalcGlobalColorDiff(&P0, &P1);
    const flt64V4 ps = psnr.calcPicPSNR(&P0, &P1);
    const flt64V4 ws = wspsnr.calcPicWSPSNR(&P0, &P1);
    const double iv = ivpsnr.calcPicIVPSNR(&P0, &P1, gcd);
    const flt64V4 ss = ssim.calcPicSSIM(&P0, &P1);
    const flt64V4 ms = ssim.calcPicMSSSIM(&P0, &P1);
    const double ivs = ivssim.calcPicIVSSIM(&P0, &P1);
    std::printf("{\"gcd\": [%d, %d, %d], \"psnr\": [%.17g, %.17g, %.17g], \"wspsnr\": [%.17g, %.17g, %.17g], "
                "\"ivpsnr\": %.17g, \"ssim\": [%.17g, %.17g, %.17g], \"msssim\": [%.17g, %.17g, %.17g], "
                "\"ivssim\": %.17g}\n",
                gcd[0], gcd[1], gcd[2], ps[0], ps[1], ps[2], ws[0], ws[1], ws[2], iv, ss[0], ss[1], ss[2], ms[0], ms[1],
                ms[2], ivs);
  }
  catch(const Error& e) { std::fprintf(stderr, "%s\n", e.what()); return 1; }
  return 0;
}
