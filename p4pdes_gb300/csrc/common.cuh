// common.cuh -- host-side helpers shared by the translation units.
#pragma once

#include <algorithm>
#include <mutex>

#include "kernels.cuh"

namespace fg {

Geom make_geom_box(int dim, int mx, int my, int mz, const double xmin[3], const double xmax[3],
                   double cx, double cy, double cz);
int sm_count();

}  // namespace fg
