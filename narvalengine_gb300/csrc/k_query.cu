// Integrator::Li over caller rays and Scene::intersectScene queries.
#include "kernels.cuh"

namespace nedev {

__global__ void k_li(const __grid_constant__ DScene s, PathParams P, nerng::PathKey base, const ne_ray* __restrict__ rays,
                     const ne_path_key* __restrict__ keys, size_t n, uint32_t first_dim, float* __restrict__ out,
                     uint32_t* err) {
  Ctx<K_GENERAL> c{s, Sampler{}, Counters{0, 0, 0, 0}, err};
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    nerng::PathKey k = base;
    k.pixel = keys[i].pixel;
    k.sample = keys[i].sample;
    c.S.reset(k, first_dim);
    Ray r{v3(rays[i].o[0], rays[i].o[1], rays[i].o[2]), v3(rays[i].d[0], rays[i].d[1], rays[i].d[2])};
    V3 L = Li(c, P, r);
    out[3 * i + 0] = L.x;
    out[3 * i + 1] = L.y;
    out[3 * i + 2] = L.z;
  }
}

__global__ void k_closest(const __grid_constant__ DScene s, const ne_ray* __restrict__ rays, size_t n, float tmin,
                          float tmax, ne_hit* __restrict__ out, uint32_t* err) {
  Ctx<K_GENERAL> c{s, Sampler{}, Counters{0, 0, 0, 0}, err};
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    Ray r{v3(rays[i].o[0], rays[i].o[1], rays[i].o[2]), v3(rays[i].d[0], rays[i].d[1], rays[i].d[2])};
    Hit h = emptyHit();
    bool did = intersectScene(c, r, h, tmin, tmax);
    ne_hit o;
    o.hit = did ? 1 : 0;
    o.pad = 0;
    if (did) {
      o.t_near = h.tNear; o.t_far = h.tFar;
      o.point[0] = h.hitPoint.x; o.point[1] = h.hitPoint.y; o.point[2] = h.hitPoint.z;
      o.normal[0] = h.normal.x; o.normal[1] = h.normal.y; o.normal[2] = h.normal.z;
      o.instance = h.inst; o.primitive = h.prim;
    } else {
      o.t_near = 0; o.t_far = 0;
      o.point[0] = o.point[1] = o.point[2] = 0;
      o.normal[0] = o.normal[1] = o.normal[2] = 0;
      o.instance = -1; o.primitive = -1;
    }
    out[i] = o;
  }
}


}  // namespace nedev

using namespace nedev;

cudaError_t ne_launch_li(int blocks, cudaStream_t st, const DScene& s, PathParams P, nerng::PathKey base,
                         const ne_ray* rays, const ne_path_key* keys, size_t n, uint32_t first_dim, float* out,
                         uint32_t* err) {
  k_li<<<blocks, kThreads, 0, st>>>(s, P, base, rays, keys, n, first_dim, out, err);
  return cudaGetLastError();
}

cudaError_t ne_launch_closest(int blocks, cudaStream_t st, const DScene& s, const ne_ray* rays, size_t n, float tmin,
                              float tmax, ne_hit* out, uint32_t* err) {
  k_closest<<<blocks, kThreads, 0, st>>>(s, rays, n, tmin, tmax, out, err);
  return cudaGetLastError();
}
