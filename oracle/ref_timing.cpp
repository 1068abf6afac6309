// Test-infrastructure timing driver around the reference QMIV metric library (pmbb-ivqm): the
// CPU baseline that bench.py reports beside the GPU numbers. Not product code; compiled by
// oracle/build_ref.sh against the reference's own sources.
//
// It runs the application's per-frame steps in the application's order with the application's
// processor set-up (apps/QMIV/src/xAppQMIV.cpp:593-650 createProcessors, :661-751
// processAllFrames, :771-830 preprocessFrames: exact-component check, margin extension on the
// thread-pool interface, interleaving for IV-PSNR; GCD; SCP; then the requested metrics, IV-PSNR on
// the interleaved pictures as with -ilp 1) and times each step per frame, like the application's
// -v 3 "AvgTime" lines. It exists because the application itself does not build on every host: its
// processor identification (libs/pmbb-base/src/xProcInfo.cpp) is x86-only, while the metric
// library has portable code paths.
//
// Usage:
//   qmiv_ref_timing -w W -h H -bd BD -cf 420|444 -i0 pic0.yuv -i1 pic1.yuv [-f frames] [-sr 2]
//                   [-erp] [-lat 180] [-lon 360] [-nth N (-1: all hardware threads)]
//                   [-ml psnr,wspsnr,ivpsnr,ssim,msssim,ivssim]
// Prints one JSON line: {"frames": F, "threads": T, "avg_ms": {"PREPROC": ..., "GCD": ..., ...}}

#include "xPic.h"
#include "xSeq.h"
#include "xThreadPool.h"
#include "xIVPSNR.h"
#include "xSSIM.h"
#include "xGlobClrDiff.h"
#include "xShftCompPic.h"
#include "xCorrespPixelShift.h"

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <thread>

using namespace PMBB_NAMESPACE;

namespace {

struct Args {
  int w = 0, h = 0, bd = 8, cf = 420, frames = 1, sr = 2, nth = -1, lat = 180, lon = 360;
  bool erp = false;
  std::string i0, i1, ml = "psnr,wspsnr,ivpsnr";
};

bool parse(int argc, char** argv, Args& a)
{
  for(int i = 1; i < argc; i++)
  {
    std::string k = argv[i];
    auto next = [&](void) -> const char* { if(i + 1 >= argc) { std::exit(2); } return argv[++i]; };
    if     (k == "-w"  ) a.w      = std::atoi(next());
    else if(k == "-h"  ) a.h      = std::atoi(next());
    else if(k == "-bd" ) a.bd     = std::atoi(next());
    else if(k == "-cf" ) a.cf     = std::atoi(next());
    else if(k == "-f"  ) a.frames = std::atoi(next());
    else if(k == "-sr" ) a.sr     = std::atoi(next());
    else if(k == "-nth") a.nth    = std::atoi(next());
    else if(k == "-lat") a.lat    = std::atoi(next());
    else if(k == "-lon") a.lon    = std::atoi(next());
    else if(k == "-erp") a.erp    = true;
    else if(k == "-ml" ) a.ml     = next();
    else if(k == "-i0" ) a.i0     = next();
    else if(k == "-i1" ) a.i1     = next();
    else { std::fprintf(stderr, "unknown arg %s\n", k.c_str()); return false; }
  }
  return a.w > 0 && a.h > 0 && !a.i0.empty() && !a.i1.empty();
}

using tClk = std::chrono::steady_clock;
double ms_since(tClk::time_point t) { return std::chrono::duration<double, std::milli>(tClk::now() - t).count(); }

} // namespace

int main(int argc, char** argv)
{
  Args a;
  if(!parse(argc, argv, a)) { std::fprintf(stderr, "bad arguments\n"); return 2; }
  std::map<std::string, bool> on;
  for(size_t b = 0; b <= a.ml.size();)
  {
    size_t e = a.ml.find(',', b);
    if(e == std::string::npos) { e = a.ml.size(); }
    on[a.ml.substr(b, e - b)] = true;
    b = e + 1;
  }
  const bool psnr = on["psnr"], wspsnr = on["wspsnr"], ivpsnr = on["ivpsnr"];
  const bool ssim = on["ssim"], msssim = on["msssim"], ivssim = on["ivssim"];
  const bool calc_psnrs = psnr || wspsnr || ivpsnr, calc_ssims = ssim || msssim || ivssim;
  const bool calc_gcd = ivpsnr || ivssim, calc_scp = ivssim; // xAppQMIV.cpp:316-322

  const int32V2 Size(a.w, a.h);
  const int32   Margin = xRoundUpToNearestMultiple(a.sr, 2); // xAppQMIV.cpp:330
  xSeq Seq0(Size, a.bd, (eCrF)a.cf), Seq1(Size, a.bd, (eCrF)a.cf);
  if(!Seq0.openFile(a.i0, xSeqBase::eMode::Read)) { std::fprintf(stderr, "cannot open %s\n", a.i0.c_str()); return 1; }
  if(!Seq1.openFile(a.i1, xSeqBase::eMode::Read)) { std::fprintf(stderr, "cannot open %s\n", a.i1.c_str()); return 1; }
  xPicP P[2] = { xPicP(Size, a.bd, Margin), xPicP(Size, a.bd, Margin) };
  xPicI I[2] = { xPicI(Size, a.bd, Margin), xPicI(Size, a.bd, Margin) };
  xPicP SCP[2] = { xPicP(Size, a.bd, Margin), xPicP(Size, a.bd, Margin) };

  const int nth = a.nth > 0 ? a.nth : (int)std::thread::hardware_concurrency(); // xAppQMIV.cpp:461-464
  xThreadPool Pool; Pool.create(nth, a.h + 1);
  xThreadPoolInterface TPI; TPI.init(&Pool, 4, 4);

  const int32V4 W = xCorrespPixelShiftPrms::c_DefaultCmpWeights;
  const flt32V4 Unc = xGlobClrDiffPrms::c_DefaultUnntcbCoef;
  xGlobClrDiffProc ProcGCD; ProcGCD.setUnntcbCoef(Unc); ProcGCD.initThreadPool(&Pool, a.h + 1);
  xShftCompPicProc ProcSCP; ProcSCP.setSearchRange(a.sr); ProcSCP.setCmpWeightsSearch(W); ProcSCP.setCmpWeightsAverage(W);
  ProcSCP.initThreadPool(&Pool, a.h + 1);
  xIVPSNR ProcPSNR;
  if(calc_psnrs)
  {
    ProcPSNR.setSearchRange(a.sr); ProcPSNR.setCmpWeightsSearch(W); ProcPSNR.setCmpWeightsAverage(W); ProcPSNR.setUnntcbCoef(Unc);
    ProcPSNR.initThreadPool(&Pool, a.h + 1);
    ProcPSNR.initRowBuffers(a.h);
    if(a.erp) { ProcPSNR.initWS(true, a.w, a.h, a.bd, a.lon, a.lat); }
  }
  xIVSSIM ProcSSIM;
  if(calc_ssims)
  {
    ProcSSIM.create(Size, a.bd, Margin, true);
    ProcSSIM.setSearchRange(a.sr); ProcSSIM.setCmpWeightsSearch(W); ProcSSIM.setCmpWeightsAverage(W); ProcSSIM.setUnntcbCoef(Unc);
    ProcSSIM.initThreadPool(&Pool, a.h + 1);
    ProcSSIM.initRowBuffers(a.h);
  }

  std::map<std::string, double> tot;
  volatile double sink = 0;
  for(int f = 0; f < a.frames; f++)
  {
    if(!Seq0.readFrame(&P[0]) || !Seq1.readFrame(&P[1])) { std::fprintf(stderr, "read error frame %d\n", f); return 1; }
    auto t = tClk::now();
    bool Exact[3];
    for(int c = 0; c < 3; c++) { Exact[c] = P[0].equalCmp(&P[1], (eCmp)c); }
    for(int i = 0; i < 2; i++) { TPI.addWaitingTask([&P, i](int32) { P[i].extend(); }); }
    TPI.waitUntilTasksFinished(2);
    if(ivpsnr)
    {
      for(int i = 0; i < 2; i++) { TPI.addWaitingTask([&P, &I, i](int32) { I[i].rearrangeFromPlanar(&P[i]); }); }
      TPI.waitUntilTasksFinished(2);
    }
    tot["PREPROC"] += ms_since(t);
    int32V4 GCD = { 0, 0, 0, 0 };
    t = tClk::now();
    if(calc_gcd) { GCD = ProcGCD.CalcGlobalColorDiff(&P[0], &P[1]); }
    tot["GCD"] += ms_since(t);
    t = tClk::now();
    if(calc_scp) { ProcSCP.GenShftCompPics(&SCP[1], &SCP[0], &P[1], &P[0], GCD); }
    tot["SCP"] += ms_since(t);
    if(psnr)   { t = tClk::now(); sink += ProcPSNR.calcPicPSNR(&P[0], &P[1])[0];       tot["PSNR"]   += ms_since(t); }
    if(wspsnr) { t = tClk::now(); sink += ProcPSNR.calcPicWSPSNR(&P[0], &P[1])[0];     tot["WSPSNR"] += ms_since(t); }
    if(ivpsnr) { t = tClk::now(); sink += ProcPSNR.calcPicIVPSNR(&I[0], &I[1], GCD);   tot["IVPSNR"] += ms_since(t); }
    if(ssim)   { t = tClk::now(); sink += ProcSSIM.calcPicSSIM(&P[0], &P[1])[0];       tot["SSIM"]   += ms_since(t); }
    if(msssim) { t = tClk::now(); sink += ProcSSIM.calcPicMSSSIM(&P[0], &P[1])[0];     tot["MSSSIM"] += ms_since(t); }
    if(ivssim) { t = tClk::now(); sink += ProcSSIM.calcPicIVSSIM(&P[0], &P[1], &SCP[0], &SCP[1]); tot["IVSSIM"] += ms_since(t); }
    (void)Exact;
  }
  std::printf("{\"frames\": %d, \"threads\": %d, \"avg_ms\": {", a.frames, nth);
  bool first = true;
  for(auto& kv : tot) { std::printf("%s\"%s\": %.4f", first ? "" : ", ", kv.first.c_str(), kv.second / a.frames); first = false; }
  std::printf("}, \"check\": %.17g}\n", (double)sink);
  TPI.uininit();
  Pool.destroy();
  return 0;
}
