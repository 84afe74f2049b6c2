// FP64 oracle renderer: the megakernel integrator (megakernel.cuh, tracer_dev.cuh) compiled with
// `real` = double.  The same estimator as the float renderers -- the reference's BSDFs, lights,
// textures, sampler draw order and quirks -- evaluated in double with exact square roots and the
// reference's double comparisons, traversing the binary LBVH; every film splat goes to the FP64
// film.  It renders the high-spp references that images report their RMSE against.
#define LTS_REAL double

#include <cuda_runtime.h>

#include <algorithm>
#include <string>

#include "dev_common.cuh"
#include "dev_math.cuh"
#include "tracer.cuh"
#include "tracer_dev.cuh"
#include "megakernel.cuh"

namespace lts {

std::string render64_launch(const SceneView& sv, const RenderParams& rp, int nleaf, bool record, cudaStream_t s) {
    static bool consts = false;  // this translation unit's copies of the texture tables
    if (!consts) {
        unsigned char p2[512];
        const float* mc = nullptr;
        texture_tables(p2, &mc);
        cudaError_t e = cudaMemcpyToSymbol(c_perm, p2, 512);
        if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_marble, mc, 30 * sizeof(float));
        if (e != cudaSuccess) return std::string("render64 tables: ") + cudaGetErrorString(e);
        consts = true;
    }
    SceneView v = sv;
    v.wnodes = nullptr;  // binary traversal in double
    v.wtris = nullptr;
    v.inst = nullptr;  // the flat binary tree holds every instance's triangles
    v.ninst = 0;
    const dim3 block(kBX, kBY);
    dim3 grid((rp.x1 - rp.x0 + kBX - 1) / kBX, (rp.y1 - rp.y0 + kBY - 1) / kBY);
    // one block per pixel tile leaves most SMs idle on the small high-spp crops this renderer
    // draws: split the samples over z until there are ~16 blocks per SM
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long tiles = (long)grid.x * grid.y;
    grid.z = (unsigned)std::max(1L, std::min<long>({(long)rp.spp, (16L * sms + tiles - 1) / tiles, 65535L}));
    if (record)
        k_pathtrace<true><<<grid, block, 0, s>>>(v, rp, nleaf);
    else
        k_pathtrace<false><<<grid, block, 0, s>>>(v, rp, nleaf);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? std::string() : std::string("render64: ") + cudaGetErrorString(e);
}

}  // namespace lts
