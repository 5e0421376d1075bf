// Host-side geometry and request checks shared by the allocating entry points
// (gnc_api.cu) and the allocation-free one (gnc_noalloc.cu), so the two cannot
// drift apart.  Both files are compiled with -ffp-contract=off: the float
// expressions below are evaluated exactly as written, as the reference's host
// code evaluates them.
#pragma once

#include <math.h>

#include <cmath>
#include <cstddef>

#include "../../include/guanaco_gb300.h"
#include "gnc_common.cuh"

namespace gnc {

// Per-tilt backprojection geometry of src/libguanaco/reconstructor.cpp:35-47
// (float arithmetic, std::cos/std::sin of a float); *offset receives the
// detector offset of a row with rotation centre `centre`.
inline TiltGeom tilt_geometry(float theta, float centre, size_t num_angles, float *offset) {
  const double output_scale = M_PI / (double)(2 * num_angles);
  const float cos_angle = std::cos(theta);
  const float sin_angle = std::sin(theta);
  const float det_x0 = -centre * cos_angle;
  const float det_y0 = -centre * sin_angle;
  const float ray_length = std::sqrt(cos_angle * cos_angle + sin_angle * sin_angle);
  const float d = cos_angle * cos_angle + sin_angle * sin_angle;
  TiltGeom g;
  *offset = (det_y0 * (-sin_angle) - det_x0 * cos_angle) / d;
  g.scale = (float)(output_scale * ray_length / std::abs(d));
  g.cos_a = cos_angle / d;
  g.sin_a = sin_angle / d;
  g.pad = 0.f;
  return g;
}

// Slab map of reconstructor.cpp:28-32 / reconstructor.cu:253-256: defocus
// coordinate = height * dscale + doffset (dscale uses D, not D - 1).
inline void defocus_scale(size_t num_defocus, float pixel_size, float min_defocus,
                          float max_defocus, float *dscale, float *doffset) {
  const float ds =
      num_defocus > 1 ? (float)num_defocus * pixel_size / (max_defocus - min_defocus) : 0.0f;
  *dscale = ds;
  *doffset = -ds * (min_defocus / pixel_size);
}

// guanaco::Config::is_valid (config.h:66-75) and BP::launch's assert
// (reconstructor.cu:250) for the single-slice entry points, plus the sizes the
// device path is built for.  GNC_OK, GNC_ERR_INVALID_ARGUMENT (the asserted
// condition in the message), or GNC_ERR_UNSUPPORTED; `who` prefixes the message.
int config_check(const gnc_config *c, const char *who);

}  // namespace gnc
