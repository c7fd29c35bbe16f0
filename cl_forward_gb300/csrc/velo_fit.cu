// velo_fit.cu -- straight-line fit of every output track (x and y linear in
// z, least squares), the stage that follows the search in the pipeline the
// reference's input files come from (their track records carry a 4-float
// header; KernelDefinitions.h:25 defines the pixel weight PARAM_W, unused by
// the search).  Hits are weighted equally by PARAM_W = 3966.94 / mm^2, so the
// weight scales chi2 only.
//
// One CTA per event, one thread per track; sums in double so the result does
// not depend on the order of the hits.
#include <cuda_runtime.h>

#include "velo_internal.h"

namespace velo {
namespace {

constexpr double kPixelWeight = 3966.94;   // PARAM_W, KernelDefinitions.h:25

__global__ void fit_tracks_kernel(const uint8_t* input, const uint64_t* ev_offset, const uint32_t* ev_valid,
                                  const velo_track* tracks, const uint32_t* counts, const uint64_t* first,
                                  int n_events, velo_track_fit* fits) {
  const int e = blockIdx.x;
  if (e >= n_events || !ev_valid[e]) return;
  const int32_t* hdr = reinterpret_cast<const int32_t*>(input + ev_offset[e]);
  const int S = hdr[0], H = hdr[1];
  const float* x = reinterpret_cast<const float*>(hdr + 2 + 3 * S + H);
  const float* y = x + H;
  const float* z = y + H;
  const uint64_t f0 = first[e];
  for (uint32_t t = threadIdx.x; t < counts[e]; t += blockDim.x) {
    const velo_track& tr = tracks[f0 + t];
    const uint32_t n = tr.hitsNum < VELO_MAX_TRACK_SIZE ? tr.hitsNum : VELO_MAX_TRACK_SIZE;
    double s0 = 0, sz = 0, szz = 0, sx = 0, sxz = 0, sy = 0, syz = 0;
    for (uint32_t k = 0; k < n; ++k) {
      const uint32_t h = tr.hits[k];
      if (h >= (uint32_t)H) continue;
      const double zz = z[h], xx = x[h], yy = y[h];
      s0 += 1;
      sz += zz;
      szz += zz * zz;
      sx += xx;
      sxz += xx * zz;
      sy += yy;
      syz += yy * zz;
    }
    velo_track_fit out{0.f, 0.f, 0.f, 0.f, 0.f};
    const double det = s0 * szz - sz * sz;
    if (s0 >= 2 && det > 0) {
      const double tx = (s0 * sxz - sz * sx) / det, ty = (s0 * syz - sz * sy) / det;
      const double x0 = (sx - tx * sz) / s0, y0 = (sy - ty * sz) / s0;
      double chi2 = 0;
      for (uint32_t k = 0; k < n; ++k) {
        const uint32_t h = tr.hits[k];
        if (h >= (uint32_t)H) continue;
        const double rx = x[h] - (x0 + tx * z[h]), ry = y[h] - (y0 + ty * z[h]);
        chi2 += kPixelWeight * (rx * rx + ry * ry);
      }
      const double ndf = 2.0 * s0 - 4.0;
      out.x0 = (float)x0;
      out.tx = (float)tx;
      out.y0 = (float)y0;
      out.ty = (float)ty;
      out.chi2_ndf = ndf > 0 ? (float)(chi2 / ndf) : 0.f;
    }
    fits[f0 + t] = out;
  }
}

}  // namespace

int launch_fit_tracks(const uint8_t* input, const uint64_t* ev_offset, const uint32_t* ev_valid,
                      const velo_track* tracks, const uint32_t* counts, const uint64_t* first, int n_events,
                      velo_track_fit* fits, void* stream) {
  if (n_events <= 0) return 0;
  fit_tracks_kernel<<<n_events, 128, 0, (cudaStream_t)stream>>>(input, ev_offset, ev_valid, tracks, counts, first,
                                                                n_events, fits);
  return (int)cudaGetLastError();
}

}  // namespace velo
