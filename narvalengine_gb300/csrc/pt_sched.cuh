// Regrouped path kernel: the integrator of pt_device.cuh as a per-lane resumable state
// machine, scheduled warp by warp.
//
// In the straight kernel (k_paths) a warp runs 32 paths to completion and waits for the
// longest one; inside a path the delta- and ratio-tracking loops of GridMedia::sample /
// GridMedia::Tr (materials/GridMedia.cpp:45-99) run different trip counts on every lane.
// Here each lane keeps its path as explicit state (program counter `pc` plus the
// variables live across the reference's loops) and the warp alternates between two
// phases chosen by ballot:
//   * tracking: every lane that is inside a tracking walk performs one step (draw,
//     advance, trilinear lookup, decide), all lanes issuing their density lookup together;
//   * transition: every other lane runs the straight-line code between walks (scene
//     queries, BSDF and light sampling, throughput updates) until it enters the next walk
//     or finishes its path.
// A lane whose path finishes takes the next work item at once (warp-aggregated atomic),
// so no lane idles while others finish long paths. The arithmetic of every step is that
// of pt_device.cuh in the same order, and each path draws the same random numbers
// (they are indexed by (pixel, sample, draw)), so results are bit-identical to k_paths
// and to the CPU oracle.
#pragma once
#include "pt_device.cuh"

namespace nedev {

enum : uint32_t {
  PC_IDLE = 0,
  PC_CAMERA,
  PC_BOUNCE,
  PC_AFTER_DELTA,
  PC_MEDIUM_AFTER_NEE,
  PC_SURFACE_AFTER_NEE,
  PC_RR,
  PC_NEE_START,
  PC_NEE_VIS_RATIO_DONE,
  PC_NEE_BSDF,
  PC_NEE_TR_LOOP,
  PC_NEE_TR_RATIO_DONE,
  PC_NEE_TR_DONE,
  PC_NEE_END,
  PC_TRACK,
  PC_DONE,
  PC_EXHAUSTED
};

enum : uint32_t { WALK_DELTA = 0, WALK_RATIO = 1 };

// One tracking walk through a grid medium, in the medium's object space.
struct Walk {
  V3 o, d;
  float t, tFar, Tr;
  int med, inst, mat;
  int steps;
  uint32_t kind, resume;
};

// Everything a path keeps alive across the reference's loops.
struct Lane {
  uint32_t pc;
  unsigned long long idx;
  // Li (VolumetricPathIntegrator.cpp:176-300)
  V3 L, T;
  Ray incoming, scattered;
  Hit isect;
  int b, passes;
  V3 sampledT, phaseRatio, ls;
  // uniformSampleOneLight / estimateDirect (VolumetricPathIntegrator.cpp:74-174)
  uint32_t neeRet;
  V3 neeD;
  int light;
  uint32_t lightInst;
  float lightPdfSel, lightPdf, scatPdf, weight;
  bool surface, found;
  V3 Ld, Li, f, woD;
  // intersectTr (VolumetricPathIntegrator.cpp:10-32)
  Ray trRay;
  V3 trTr;
  int seg;
  float walkResult;
  Walk w;
};

// Starts a ratio-tracking walk for GridMedia::Tr(ray, isect) (GridMedia.cpp:45-53).
NE_D void startRatio(const DScene& s, Lane& st, const Ray& rayWcs, const Hit& h, int med, uint32_t resume) {
  Ray r = transformRay(rayWcs, s.instances[h.inst].ocs);
  st.w.o = r.at(h.tNear);
  st.w.d = r.d;
  st.w.tFar = h.tFar - h.tNear;
  st.w.t = 0;
  st.w.Tr = 1;
  st.w.med = med;
  st.w.inst = h.inst;
  st.w.mat = -1;
  st.w.steps = 0;
  st.w.kind = WALK_RATIO;
  st.w.resume = resume;
  st.pc = PC_TRACK;
}

// One iteration of the loops of GridMedia::sample (GridMedia.cpp:80-97) or GridMedia::Tr
// (GridMedia.cpp:56-67). On leaving the walk the lane's pc becomes w.resume with the
// walk's result in sampledT/scattered (delta) or walkResult (ratio).
template <uint32_t K>
NE_D void walkStep(Ctx<K>& c, Lane& st) {
  Walk& w = st.w;
  const DMedium& M = c.s.media[w.med];
  float u = c.S.random();
  w.t -= (nefm::log(1 - u) * M.inv_max_density) / M.mu;
  bool leave = false;
  if (w.t >= w.tFar) {
    if (w.kind == WALK_DELTA)
      st.sampledT = v3(1, 1, 1);
    else
      st.walkResult = w.Tr;
    leave = true;
  } else {
    float density = sampleAt(c, M, Ray{w.o, w.d}, w.t);
    if (w.kind == WALK_DELTA) {
      float ra = c.S.random();
      if (density * M.inv_max_density > ra) {
        Ray sc;
        sc.o = w.o + w.t * w.d;
        sc.d = bsdfSample<K>(c.s.materials[w.mat], w.d, v3(0, 1, 0), c.S);
        st.scattered = transformRay(sc, c.s.instances[w.inst].wcs);
        st.sampledT = ld3(M.sigma_s) / ld3(M.sigma_t);
        leave = true;
      }
    } else {
      float x = density * M.inv_max_density;
      w.Tr *= 1 - ((0.0f < x) ? x : 0.0f);
      if (w.Tr < 0.1f) {
        float q = (0.05f < 1.0f - w.Tr) ? (1.0f - w.Tr) : 0.05f;
        if (c.S.random() < q) {
          st.walkResult = 0.0f;
          leave = true;
        } else {
          w.Tr /= 1 - q;
        }
      }
    }
  }
  if (!leave && ++w.steps >= kMaxTrackSteps) {
    if (w.kind == WALK_DELTA)
      st.sampledT = v3(1, 1, 1);
    else
      st.walkResult = w.Tr;
    leave = true;
  }
  if (leave) st.pc = w.resume;
}

}  // namespace nedev

namespace nedev {

// Starts a camera path (core/OfflineEngine.cpp:64-67, core/Camera.cpp:140-144).
NE_D void startPath(const DScene& s, Sampler& S, Lane& st, const nerng::PathKey& base, uint32_t pixel,
                    uint32_t sample) {
  uint32_t W = (uint32_t)s.width;
  uint32_t x = pixel % W, y = pixel / W;
  nerng::PathKey k = base;
  k.pixel = pixel;
  k.sample = sample;
  S.reset(k, 0);
  float u = (float)((float)(int)x + S.random()) / (float)s.width;
  float v = (float)((float)(int)y + S.random()) / (float)s.height;
  st.incoming = cameraRay(s.camera, u, v, S);
  st.L = v3(0, 0, 0);
  st.T = v3(1, 1, 1);
  st.isect = emptyHit();
  st.b = 0;
  st.passes = 0;
  st.pc = PC_BOUNCE;
}

// Runs the straight-line code of Li, uniformSampleOneLight, estimateDirect, visibilityTr
// and intersectTr (integrators/VolumetricPathIntegrator.cpp:10-300) from st.pc until the
// lane enters a tracking walk (PC_TRACK) or its path ends (PC_DONE).
template <uint32_t K>
NE_NI void transition(Ctx<K>& c, Lane& st, const PathParams& P) {
  const DScene& s = c.s;
  const float inf = __int_as_float(0x7f800000);
  for (;;) {
    switch (st.pc) {
      case PC_BOUNCE: {
        if (st.b >= P.bounces) { st.pc = PC_DONE; return; }
        bool did = intersectScene(c, st.incoming, st.isect, kEps12F, inf);
        if (isBlack(st.T)) { st.pc = PC_DONE; return; }
        const DMaterial* mat = did ? matOf(s, st.isect.prim) : nullptr;
        if ((K & FT_VOLBSDF) && did && mat && mat->bsdf == NE_BSDF_VOLUME) {
          st.incoming.o = st.incoming.at(st.isect.tNear);
          st.isect.tFar = st.isect.tFar - st.isect.tNear;
          st.isect.tNear = 0;
          const DMedium& M = s.media[mat->medium];
          if ((K & FT_GRID) && M.type == NE_MEDIUM_GRID) {
            // GridMedia::sample (GridMedia.cpp:71-79): scattered starts as the incoming ray
            st.scattered = st.incoming;
            Ray r = transformRay(st.incoming, s.instances[st.isect.inst].ocs);
            st.w.o = r.o;
            st.w.d = r.d;
            st.w.t = st.isect.tNear;
            st.w.tFar = st.isect.tFar;
            st.w.med = mat->medium;
            st.w.inst = st.isect.inst;
            st.w.mat = s.prims[st.isect.prim].material;
            st.w.steps = 0;
            st.w.kind = WALK_DELTA;
            st.w.resume = PC_AFTER_DELTA;
            st.pc = PC_TRACK;
            return;
          }
          st.scattered = Ray{v3(0, 0, 0), v3(0, 0, 0)};
          st.sampledT = (K & FT_HOMOG) ? homogSample(c, M, st.incoming, st.scattered, st.isect) : v3(1, 1, 1);
          st.pc = PC_AFTER_DELTA;
          break;
        }
        if (st.b == 0) {
          if (did && mat && mat->light >= 0) {
            st.L = st.L + st.T * lightLi(s.lights[mat->light]);
          } else {
            for (uint32_t li = 0; li < s.n_light_instances; li++) {
              const DInstance& inst = s.instances[s.n_instances + li];
              const DModel& lm = s.models[inst.model];
              for (uint32_t k = 0; k < lm.mat_count; k++) {
                const DMaterial& mm = s.materials[s.model_materials[lm.mat_begin + k]];
                st.L = st.L + st.T * lightLe<K>(s.lights[mm.light], inst.ocs, st.incoming.d);
              }
            }
          }
        }
        if (!did || !mat || mat->bsdf == NE_BSDF_NONE) { st.pc = PC_DONE; return; }
        st.neeD = st.incoming.d;
        st.neeRet = PC_SURFACE_AFTER_NEE;
        st.pc = PC_NEE_START;
        break;
      }
      case PC_AFTER_DELTA: {
        const DMaterial& mat = *matOf(s, st.isect.prim);
        if (areAllOne(st.sampledT)) {
          st.incoming.o = st.incoming.at(st.isect.tFar + 0.01f);
          if (++st.passes >= kMaxPassThrough) { st.pc = PC_DONE; return; }
          st.pc = PC_BOUNCE;
          break;
        }
        st.T = st.T * st.sampledT;
        V3 phaseFr = bsdfEval<K>(s, mat, st.incoming, st.scattered.d, st.isect);  // VolumeBSDF: (p, p, p)
        float phasePdf = phaseFr.x;                                                   // and its pdf p
        if (isBlack(phaseFr) || phasePdf == 0.f) { st.pc = PC_DONE; return; }
        st.phaseRatio = phaseFr / phasePdf;
        st.neeD = st.scattered.d;
        st.neeRet = PC_MEDIUM_AFTER_NEE;
        st.pc = PC_NEE_START;
        break;
      }
      case PC_MEDIUM_AFTER_NEE:
        st.T = st.T * st.phaseRatio;
        st.L = st.L + st.T * st.ls;
        st.incoming = st.scattered;
        st.pc = PC_RR;
        break;
      case PC_SURFACE_AFTER_NEE: {
        const DMaterial& mat = *matOf(s, st.isect.prim);
        st.L = st.L + st.T * st.ls;
        Ray sc;
        sc.o = st.isect.hitPoint;
        sc.d = bsdfSample<K>(mat, st.incoming.d, st.isect.normal, c.S);
        float pdf = bsdfPdf<K>(mat, st.incoming.d, sc.d, st.isect.normal);
        V3 fr = bsdfEval<K>(s, mat, st.incoming, sc.d, st.isect);
        if (isBlack(fr) || pdf == 0.f) { st.pc = PC_DONE; return; }
        st.T = st.T * ((fr * absDot(st.incoming.d, st.isect.normal)) / pdf);
        st.incoming = sc;
        st.pc = PC_RR;
        break;
      }
      case PC_RR:
        if (P.rr && st.b > P.rr_after) {
          float mx = maxc(st.T);
          if (mx < 0.01f) {
            float q = gmax(0.05f, 1.0f - mx);
            if (c.S.random() < q) { st.pc = PC_DONE; return; }
            st.T = st.T / (1.0f - q);
          }
        }
        st.b++;
        st.pc = PC_BOUNCE;
        break;
      case PC_NEE_START: {
        // uniformSampleOneLight (VolumetricPathIntegrator.cpp:159-174)
        float r = c.S.random();
        uint32_t nL = s.n_light_instances;
        if (nL == 0) { st.ls = v3(0, 0, 0); st.pc = st.neeRet; break; }
        int i = (int)((float)nL * r);
        st.lightPdfSel = 1.0f / (float)nL;
        st.lightInst = s.n_instances + (uint32_t)i;
        const DModel& m = s.models[s.instances[st.lightInst].model];
        if (m.light_count == 0) { st.ls = v3(0, 0, 0); st.pc = st.neeRet; break; }
        c.S.random();
        float r2 = c.S.random();
        int k = (int)((float)m.light_count * r2);
        st.light = s.materials[s.prims[m.light_begin + k].material].light;
        // estimateDirect, light sampling branch (VolumetricPathIntegrator.cpp:75-111)
        const DLight& light = s.lights[st.light];
        const DInstance& lin = s.instances[st.lightInst];
        const DMaterial& mat = *matOf(s, st.isect.prim);
        st.Ld = v3(0, 0, 0);
        Ray wo{v3(0, 0, 0), v3(0, 0, 0)};
        st.lightPdf = 0;
        st.scatPdf = 0;
        st.Li = sampleLi<K>(s, light, st.isect, lin, wo, st.lightPdf, c.S);
        st.woD = wo.d;
        st.f = v3(0, 0, 0);
        st.surface = !(mat.medium >= 0);
        st.pc = PC_NEE_BSDF;
        if (st.lightPdf > 0 && !isBlack(st.Li)) {
          if (st.surface) {
            st.f = bsdfEval<K>(s, mat, Ray{st.incoming.o, st.neeD}, st.woD, st.isect) * fabsf(dot(st.woD, st.isect.normal));
            st.scatPdf = bsdfPdf<K>(mat, st.neeD, st.woD, st.isect.normal);
          } else {
            st.f = bsdfEval<K>(s, mat, Ray{st.incoming.o, st.neeD}, st.woD, st.isect);
            st.scatPdf = st.f.x;
          }
          if (!isBlack(st.f)) {
            V3 pointOnLight = samplePointOnSurface<K>(s, light.primitive, st.isect, lin.wcs, c.S);
            // visibilityTr (VolumetricPathIntegrator.cpp:34-72)
            Ray ray{st.isect.hitPoint, pointOnLight - st.isect.hitPoint};
            Hit vh = emptyHit();
            bool hit = intersectScene(c, ray, vh, kEps3F, inf);
            V3 vis = v3(1, 1, 1);
            if (hit) {
              const DMaterial* vm = matOf(s, vh.prim);
              if (!vm) {
                vis = v3(0, 0, 0);
              } else if (vm->light < 0) {
                if (vm->medium >= 0) {
                  const DMedium& VM = s.media[vm->medium];
                  if ((K & FT_GRID) && VM.type == NE_MEDIUM_GRID) {
                    startRatio(s, st, ray, vh, vm->medium, PC_NEE_VIS_RATIO_DONE);
                    return;
                  }
                }
                vis = v3(0, 0, 0);
              }
            }
            st.Li = st.Li * vis;
            if (!isBlack(st.Li)) {
              float weight = powerHeuristic(st.lightPdf, st.scatPdf);
              st.Ld = st.Ld + ((st.f * st.Li) * weight) / st.lightPdf;
            }
          }
        }
        break;
      }
      case PC_NEE_VIS_RATIO_DONE:
        // the transmittance is computed and discarded: any non-emitter hit returns 0
        st.Li = st.Li * v3(0, 0, 0);
        if (!isBlack(st.Li)) {
          float weight = powerHeuristic(st.lightPdf, st.scatPdf);
          st.Ld = st.Ld + ((st.f * st.Li) * weight) / st.lightPdf;
        }
        st.pc = PC_NEE_BSDF;
        break;
      case PC_NEE_BSDF: {
        // estimateDirect, BSDF sampling branch (VolumetricPathIntegrator.cpp:113-143)
        const DMaterial& mat = *matOf(s, st.isect.prim);
        if (st.surface) {
          st.woD = bsdfSample<K>(mat, st.neeD, st.isect.normal, c.S);
          st.f = bsdfEval<K>(s, mat, Ray{st.incoming.o, st.neeD}, st.woD, st.isect);
          st.f = st.f * fabsf(dot(st.woD, st.isect.normal));
          st.scatPdf = bsdfPdf<K>(mat, st.neeD, st.woD, st.isect.normal);
        } else {
          st.f = bsdfEval<K>(s, mat, Ray{st.incoming.o, st.neeD}, st.woD, st.isect);
          st.woD = bsdfSample<K>(mat, st.neeD, v3(0, 1, 0), c.S);
          st.scatPdf = st.f.x;
        }
        st.pc = PC_NEE_END;
        if (!isBlack(st.f) && st.scatPdf > 0) {
          const DLight& light = s.lights[st.light];
          st.lightPdf = primPdf<K>(s, light.primitive, st.isect, s.instances[st.lightInst], c.S);
          if (st.lightPdf == 0) break;
          st.weight = powerHeuristic(st.scatPdf, st.lightPdf);
          st.trRay = Ray{st.isect.hitPoint, st.woD};
          st.trTr = v3(1, 1, 1);
          st.seg = 0;
          st.pc = PC_NEE_TR_LOOP;
        }
        break;
      }
      case PC_NEE_TR_LOOP: {
        // intersectTr (VolumetricPathIntegrator.cpp:10-32)
        if (st.seg >= kMaxTrSegments) { st.found = false; st.pc = PC_NEE_TR_DONE; break; }
        Hit th = emptyHit();
        bool hitSurface = intersectScene(c, st.trRay, th, kEps3F, inf);
        const DMaterial* tm = hitSurface ? matOf(s, th.prim) : nullptr;
        int m = tm ? tm->medium : -1;
        if (m >= 0) {
          const DMedium& TM = s.media[m];
          if ((K & FT_GRID) && TM.type == NE_MEDIUM_GRID) {
            startRatio(s, st, st.trRay, th, m, PC_NEE_TR_RATIO_DONE);
            return;
          }
          if (K & FT_HOMOG) st.trTr = st.trTr * homogTr(TM, th.tFar - th.tNear);
        }
        if (!hitSurface) { st.found = false; st.pc = PC_NEE_TR_DONE; break; }
        if (m >= 0) { st.found = true; st.pc = PC_NEE_TR_DONE; break; }
        if (sameBits(th.hitPoint, st.trRay.o)) { st.found = false; st.pc = PC_NEE_TR_DONE; break; }
        st.trRay.o = th.hitPoint;
        st.seg++;
        break;
      }
      case PC_NEE_TR_RATIO_DONE:
        st.trTr = st.trTr * v3(st.walkResult, st.walkResult, st.walkResult);
        st.found = true;
        st.pc = PC_NEE_TR_DONE;
        break;
      case PC_NEE_TR_DONE: {
        // VolumetricPathIntegrator.cpp:144-154
        V3 Li2 = st.found ? lightLi(s.lights[st.light]) : v3(0, 0, 0);
        if (!isBlack(Li2)) st.Ld = st.Ld + (((st.f * Li2) * st.trTr) * st.weight) / st.scatPdf;
        st.pc = PC_NEE_END;
        break;
      }
      case PC_NEE_END:
        st.ls = st.Ld / st.lightPdfSel;
        st.pc = st.neeRet;
        break;
      default:
        return;
    }
  }
}

// The regrouped persistent kernel. Work items are (pixel, sample) as in k_paths.
// trackShare: a warp keeps stepping walks while at least trackShare/32 of its live
// lanes are inside one (the rest wait); otherwise it runs transitions.
template <uint32_t K>
__device__ __forceinline__ void schedLoop(const DScene& s, const PathParams& P, const nerng::PathKey& base,
                                          unsigned long long total, uint32_t spp, uint32_t sampleOffset,
                                          uint32_t coverW, const ne_path_key* keys, float* out,
                                          unsigned long long* counter, uint32_t* err, int trackShare) {
  Ctx<K> c{s, Sampler{}, Counters{0, 0, 0, 0}, err};
  const unsigned lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  trackShare = trackShare < 1 ? 1 : (trackShare > 32 ? 32 : trackShare);
  Lane st;
  st.pc = PC_IDLE;
  for (;;) {
    // refill lanes whose path finished
    unsigned idle = __ballot_sync(0xffffffffu, st.pc == PC_IDLE);
    if (idle) {
      unsigned long long base0 = 0;
      unsigned n = __popc(idle);
      int leader = __ffs(idle) - 1;
      if ((int)lane == leader) base0 = atomicAdd(&counter[0], (unsigned long long)n);
      base0 = __shfl_sync(0xffffffffu, base0, leader);
      if (st.pc == PC_IDLE) {
        unsigned long long idx = base0 + __popc(idle & lt);
        if (idx < total) {
          uint32_t pixel, sample;
          if (keys) {
            pixel = keys[idx].pixel;
            sample = keys[idx].sample + sampleOffset;
          } else {
            uint32_t pi = (uint32_t)(idx / spp);
            sample = (uint32_t)(idx % spp) + sampleOffset;
            pixel = (pi / coverW) * (uint32_t)s.width + (pi % coverW);
          }
          st.idx = idx;
          startPath(s, c.S, st, base, pixel, sample);
        } else {
          st.pc = PC_EXHAUSTED;
        }
      }
    }
    unsigned live = __ballot_sync(0xffffffffu, st.pc != PC_EXHAUSTED);
    if (!live) break;
    unsigned tracking = __ballot_sync(0xffffffffu, st.pc == PC_TRACK);
    if (tracking && (int)__popc(tracking) * 32 >= trackShare * (int)__popc(live)) {
      // tracking phase: step walks while enough lanes are in one
      do {
        if (st.pc == PC_TRACK) walkStep(c, st);
        tracking = __ballot_sync(0xffffffffu, st.pc == PC_TRACK);
      } while (tracking && (int)__popc(tracking) * 32 >= trackShare * (int)__popc(live));
    } else {
      if (st.pc != PC_TRACK && st.pc != PC_EXHAUSTED) {
        transition(c, st, P);
        if (st.pc == PC_DONE) {
          out[3 * st.idx + 0] = st.L.x;
          out[3 * st.idx + 1] = st.L.y;
          out[3 * st.idx + 2] = st.L.z;
          st.pc = PC_IDLE;
        }
      }
    }
  }
  if (K & K_COUNT) {
    unsigned long long v[4] = {c.c.lookups, c.c.queries, c.c.nodes, c.c.tests};
#pragma unroll
    for (int k = 0; k < 4; k++) {
      unsigned long long x = v[k];
      for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
      if (lane == 0 && x) atomicAdd(&counter[1 + k], x);
    }
  }
}

}  // namespace nedev
