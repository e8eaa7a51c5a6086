// rk.cuh -- classical RK4 stage combination shared by the plain and the
// matrix-free kernels.  Same formulas as the FP64 oracle: acc collects
// k1 + 2k2 + 2k3, the next stage input is y + c dt k, and at stage 4
// y += dt/6 (acc + k4) (the new y is also the next step's stage input).
// hdt = dt / 2 and dt6 = dt / 6 come from the host (the same correctly
// rounded values; FP64 arithmetic per element is slow on this GPU).
#pragma once

namespace sgdg {

__device__ __forceinline__ void rk_stage(int stage, double dt, double hdt, double dt6, double k, double& y,
                                         double& acc, double& un) {
    switch (stage) {
        case 1: acc = k; un = y + hdt * k; break;
        case 2: acc = acc + 2.0 * k; un = y + hdt * k; break;
        case 3: acc = acc + 2.0 * k; un = y + dt * k; break;
        default: y = y + dt6 * (acc + k); un = y; break;
    }
}

}  // namespace sgdg
