// nfw_device.cuh -- elliptical NFW deflection on the device (quadrature and
// surrogate); placeholder until the NFW path lands.
#pragma once
#include "qlpix_internal.h"
namespace qlpix {
__device__ __forceinline__ void nfw_deflection(const LensRec& L, double x, double y, double& dx, double& dy)
{
    (void)L; (void)x; (void)y;
    dx = 0; dy = 0;
}
}  // namespace qlpix
