// Host-only entry points over csrc/bgk_setup.h, the case setup that bgk_create runs on the host
// before it allocates anything: scalars (SRC/hencol.F90, SRC/build.bcond.F90), obstacle mask and
// bounding box (SRC/build.obs.F90) and the reference initial state (SRC/init.F90).  Built as a
// shared library that makes no CUDA call, so tests/test_setup_host.py can compare the product's
// setup with the oracle on a machine without a GPU.
#include <cstring>
#include <string>
#include <vector>

#include "../../bgk2d_gpu_gb300/csrc/bgk_setup.h"

using namespace bgk;

// prec: 0 SINGLE (FP32 storage and arithmetic), 1 DOUBLE, 2 MIXED2 (FP32 storage, FP64 arithmetic)
extern "C" int host_setup(int lx, int ly, int tcase, double svisc, double u0, int prec, int obstacle, int radius,
                          int icoord, int jcoord, double scalars[4], int32_t *mask, int32_t bbox[5])
{
    bgk_case_desc d;
    std::memset(&d, 0, sizeof(d));
    d.lx = lx;
    d.ly = ly;
    d.tcase = tcase;
    d.svisc = svisc;
    d.u0 = u0;
    d.storage = prec == 1 ? BGK_STORE_F64 : BGK_STORE_F32;
    d.compute = prec == 0 ? BGK_COMPUTE_F32 : BGK_COMPUTE_F64;
    d.scheme = BGK_SCHEME_PINGPONG;
    d.obstacle = obstacle;
    d.radius = radius;
    d.obs_icoord = icoord;
    d.obs_jcoord = jcoord;
    d.cte_s = 0.1;
    CaseSetup cs;
    const std::string msg = prec == 0 ? setup_case<float>(d, cs) : setup_case<double>(d, cs);
    if (!msg.empty()) return 1;
    scalars[0] = cs.omega;
    scalars[1] = cs.fgrad;
    scalars[2] = cs.u00;
    scalars[3] = cs.u0;
    std::memset(mask, 0, sizeof(int32_t) * (size_t)lx * ly);
    if (!cs.obs.empty()) std::memcpy(mask, cs.obs.data(), sizeof(int32_t) * cs.obs.size());
    for (int i = 0; i < 5; ++i) bbox[i] = cs.bbox[i];
    return 0;
}

// -DTRICK1 setup (SRC/check_case.F90:173-178): 1 when accepted with the x-wall corner rule on,
// -1 when refused
extern "C" int host_trick1(int lx, int ly, int tcase)
{
    bgk_case_desc d;
    std::memset(&d, 0, sizeof(d));
    d.lx = lx;
    d.ly = ly;
    d.tcase = tcase;
    d.svisc = 0.05;
    d.u0 = 0.1;
    d.storage = BGK_STORE_F32;
    d.compute = BGK_COMPUTE_F32;
    d.scheme = BGK_SCHEME_PINGPONG;
    d.trick1 = 1;
    CaseSetup cs;
    const std::string msg = setup_case<float>(d, cs);
    return msg.empty() ? cs.corner_x : -1;
}

// the nine (0:l+1, 0:m+1) population planes of the reference initial state, in the storage kind
// (deviations, or whole populations when noshift is set)
extern "C" void host_init(int l, int m, int vortex, int prec, int noshift, void *out)
{
    const size_t n = 9 * (size_t)(l + 2) * (size_t)(m + 2);
    if (prec == 1) {
        std::vector<double> a;
        init_reference<double, double>(l, m, vortex != 0, a, noshift != 0);
        std::memcpy(out, a.data(), n * sizeof(double));
    } else {
        std::vector<float> a;
        if (prec == 2) init_reference<double, float>(l, m, vortex != 0, a, noshift != 0);
        else init_reference<float, float>(l, m, vortex != 0, a, noshift != 0);
        std::memcpy(out, a.data(), n * sizeof(float));
    }
}
