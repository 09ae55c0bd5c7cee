// Batched execution: many GaussianFilter requests (and VJPs) of uneven sizes
// and sigmas planned once and replayed as one CUDA graph.  No counterpart in
// the reference, which filters one image per generate_region call
// (src/filters/gaussian.rs:59-91).
//
// Planning:
//   1. every forward item is classified by (dimension, components, dtype,
//      radii, rounding, alignment); items of one class that the fused kernel
//      covers are merged into one persistent multi-item launch whose CTAs split
//      the union of the items' (tile, slice) units evenly;
//   2. an autotuner times, once per class key (dtype, axis-length bucket,
//      radius), the fused kernel against the per-axis passes on the class's
//      first item and keeps the faster (the "fusion depth": 3 axes in one
//      kernel, or one axis per kernel); its choices are cached process-wide;
//   3. the chosen launches (plus the VJP items' passes) are captured into a
//      CUDA graph, instantiated once; itkg_batch_run replays it on the
//      caller's stream.  The items are independent, so they are spread over
//      kLanes concurrent lanes (branches of the graph) by longest-processing-
//      time-first on an estimate of their work (voxels x taps): small volumes
//      and the tails of large ones then overlap instead of queueing.
// Scratch the captured work needs comes from graph memory nodes
// (stream-ordered allocation inside the capture).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "geom.hpp"
#include "internal.hpp"

struct itkg_batch {
  struct Fwd {
    itkg_image in, out;
    itkg_region largest, requested;
    itkg_gaussian_params prm;
  };
  struct Vjp {
    itkg_image x, ybar, xbar;
    bool has_xbar;
    itkg_gaussian_params prm;
    double* sigma_bar;  // device pointer or NULL
    int32_t flags;
  };
  std::vector<Fwd> fwd;
  std::vector<Vjp> vjp;
  int device = -1;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<std::string> plan_lines;  // human-readable plan (itkg_batch_describe)
  std::string described;
  uint64_t launches_per_run = 0;
  itkg::FusedMultiPlan* fused = nullptr;  // request tables of the multi-request launches
  itkg::Tile2DMultiPlan* tiles2d = nullptr;  // the 2-D items' multi-request tile launches
};

namespace itkg {
namespace {

// ---- autotuner ------------------------------------------------------------
// key: (dtype, comps, dim, radius x/y/z, rounding, log2 bucket of the smallest
// requested axis) -> algorithm
using TuneKey = std::tuple<int, int, int, int, int, int, int, int>;
std::mutex g_tune_mu;
std::map<TuneKey, int> g_tune;

int bucket(uint64_t n) {
  int b = 0;
  while (n > 1) {
    n >>= 1;
    ++b;
  }
  return b;
}

TuneKey key_of(const itkg_batch::Fwd& f) {
  uint64_t r[3] = {0, 0, 0};
  uint64_t mn = UINT64_MAX;
  for (int d = 0; d < f.in.dim; ++d) {
    r[d] = kernel_radius(f.prm.sigma, f.in.spacing[d]);
    mn = std::min<uint64_t>(mn, f.requested.size[d]);
  }
  return TuneKey(f.in.dtype, f.in.components, f.in.dim, (int)r[0], (int)r[1], (int)r[2],
                 f.prm.rounding, bucket(mn));
}

itkg_status time_item(itkg_batch::Fwd f, int algo, cudaStream_t s, float* ms) {
  f.prm.algorithm = algo;
  cudaEvent_t e0, e1;
  ITKG_CUDA(cudaEventCreate(&e0));
  ITKG_CUDA(cudaEventCreate(&e1));
  itkg_status st = ITKG_SUCCESS;
  // one warm-up, then the best of three
  float best = 1e30f;
  for (int it = 0; it < 4 && st == ITKG_SUCCESS; ++it) {
    cudaEventRecord(e0, s);
    st = itkg_gaussian_generate_region(&f.in, &f.largest, &f.requested, &f.prm, &f.out, s);
    cudaEventRecord(e1, s);
    if (st == ITKG_SUCCESS) {
      cudaEventSynchronize(e1);
      float t = 0.0f;
      cudaEventElapsedTime(&t, e0, e1);
      if (it > 0) best = std::min(best, t);
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *ms = best;
  return st;
}

itkg_status choose_algorithm(const itkg_batch::Fwd& f, bool tune, cudaStream_t s, int* algo) {
  if (f.prm.algorithm != ITKG_ALGO_AUTO || f.prm.arithmetic == ITKG_ARITH_PIXEL_U8) {
    *algo = f.prm.algorithm == ITKG_ALGO_AUTO ? ITKG_ALGO_PER_AXIS : f.prm.algorithm;
    return ITKG_SUCCESS;
  }
  const TuneKey k = key_of(f);
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(k);
    if (it != g_tune.end()) {
      *algo = it->second;
      return ITKG_SUCCESS;
    }
  }
  // Is a fused kernel available at all for this item?
  itkg_batch::Fwd probe = f;
  probe.prm.algorithm = ITKG_ALGO_FUSED;
  if (!tune) {
    *algo = ITKG_ALGO_AUTO;  // the per-call dispatcher decides
    return ITKG_SUCCESS;
  }
  float t_fused = 1e30f, t_axis = 1e30f, t_two = 1e30f;
  const itkg_status sf = time_item(probe, ITKG_ALGO_FUSED, s, &t_fused);
  if (sf != ITKG_SUCCESS && sf != ITKG_ERROR_UNSUPPORTED) return sf;
  const itkg_status s2 = time_item(f, ITKG_ALGO_TWO_PASS, s, &t_two);
  if (s2 != ITKG_SUCCESS && s2 != ITKG_ERROR_UNSUPPORTED) return s2;
  ITKG_TRY(time_item(f, ITKG_ALGO_PER_AXIS, s, &t_axis));
  if (sf != ITKG_SUCCESS) t_fused = 1e30f;
  if (s2 != ITKG_SUCCESS) t_two = 1e30f;
  int pick = ITKG_ALGO_PER_AXIS;
  if (t_fused <= t_axis && t_fused <= t_two) pick = ITKG_ALGO_FUSED;
  else if (t_two < t_axis) pick = ITKG_ALGO_TWO_PASS;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune[k] = pick;
  *algo = pick;
  return ITKG_SUCCESS;
}

constexpr int kLanes = 4;  // concurrent branches of the batch graph (8 measured slower)

// Work estimate of one filter over an image: voxels x taps summed over the axes.
double work_of(const itkg_image& im, const itkg_region& reg, double sigma) {
  double vox = 1.0, taps = 0.0;
  for (int d = 0; d < im.dim; ++d) {
    vox *= (double)reg.size[d];
    taps += 2.0 * (double)kernel_radius(sigma, im.spacing[d]) + 1.0;
  }
  return vox * (taps + 4.0) * (double)im.components;
}

itkg_status check_device_item(const itkg_image* im, const char* name) {
  ITKG_TRY(validate_image(im, name));
  ITKG_TRY(filter_components(im, name));
  if (im->location != ITKG_DEVICE)
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "%s: batch items take device buffers", name);
  return ITKG_SUCCESS;
}

}  // namespace
}  // namespace itkg

using namespace itkg;

extern "C" {

itkg_status itkg_batch_create(itkg_batch** out) {
  if (!out) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "out is NULL");
  *out = new itkg_batch();
  return ITKG_SUCCESS;
}

itkg_status itkg_batch_destroy(itkg_batch* b) {
  if (!b) return ITKG_SUCCESS;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  fused_multi_free(b->fused);
  tile2d_multi_free(b->tiles2d);
  delete b;
  return ITKG_SUCCESS;
}

itkg_status itkg_batch_add(itkg_batch* b, const itkg_image* input, const itkg_region* largest,
                           const itkg_region* requested, const itkg_gaussian_params* params,
                           itkg_image* output) {
  if (!b || !largest || !requested || !params)
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "NULL argument");
  if (b->exec) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "batch already planned");
  ITKG_TRY(check_device_item(input, "input"));
  ITKG_TRY(check_device_item(output, "output"));
  itkg_batch::Fwd f;
  f.in = *input;
  f.out = *output;
  f.largest = *largest;
  f.requested = *requested;
  f.prm = *params;
  b->fwd.push_back(f);
  return ITKG_SUCCESS;
}

itkg_status itkg_batch_add_vjp(itkg_batch* b, const itkg_image* x, const itkg_image* ybar,
                               const itkg_gaussian_params* params, itkg_image* xbar,
                               double* sigma_bar_device, int32_t flags) {
  if (!b || !params) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "NULL argument");
  if (b->exec) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "batch already planned");
  ITKG_TRY(check_device_item(x, "x"));
  ITKG_TRY(check_device_item(ybar, "ybar"));
  if (xbar) ITKG_TRY(check_device_item(xbar, "xbar"));
  itkg_batch::Vjp v;
  v.x = *x;
  v.ybar = *ybar;
  v.has_xbar = xbar != nullptr;
  if (xbar) v.xbar = *xbar;
  v.prm = *params;
  v.sigma_bar = sigma_bar_device;
  v.flags = flags | (sigma_bar_device ? ITKG_VJP_SIGMA_BAR_ON_DEVICE : 0);
  b->vjp.push_back(v);
  return ITKG_SUCCESS;
}

itkg_status itkg_batch_plan(itkg_batch* b, int32_t flags, void* stream) {
  if (!b) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "batch is NULL");
  if (b->exec) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "batch already planned");
  cudaStream_t user = static_cast<cudaStream_t>(stream);
  ITKG_CUDA(cudaGetDevice(&b->device));
  const bool tune = (flags & ITKG_BATCH_NO_AUTOTUNE) == 0;

  // 1. choose per-item algorithms (autotuned per class key)
  std::vector<int> algo(b->fwd.size());
  for (size_t i = 0; i < b->fwd.size(); ++i) ITKG_TRY(choose_algorithm(b->fwd[i], tune, user, &algo[i]));
  ITKG_CUDA(cudaStreamSynchronize(user));

  // 2. group fused forward items by kernel class for multi-item launches: the
  // 3-D items the fused kernel covers, and the 2-D items the tile kernel covers
  std::vector<FusedGeom> fused_geoms, tile_geoms;
  std::vector<std::vector<std::vector<float>>> fused_w, tile_w;
  std::vector<size_t> per_item;
  for (size_t i = 0; i < b->fwd.size(); ++i) {
    if (b->fwd[i].in.dim == 2 && algo[i] != ITKG_ALGO_PER_AXIS) {
      FusedGeom g;
      std::vector<std::vector<float>> w;
      if (tile2d_geom_for(b->fwd[i].in, b->fwd[i].largest, b->fwd[i].requested, b->fwd[i].prm, b->fwd[i].out, &g,
                          &w) == ITKG_SUCCESS) {
        tile_geoms.push_back(g);
        tile_w.push_back(std::move(w));
        continue;
      }
    }
    if (algo[i] == ITKG_ALGO_PER_AXIS || algo[i] == ITKG_ALGO_TWO_PASS) {
      per_item.push_back(i);
      continue;
    }
    FusedGeom g;
    std::vector<std::vector<float>> w;
    const itkg_status st = fused_geom_for(b->fwd[i].in, b->fwd[i].largest, b->fwd[i].requested,
                                          b->fwd[i].prm, b->fwd[i].out, &g, &w);
    if (st == ITKG_SUCCESS) {
      fused_geoms.push_back(g);
      fused_w.push_back(std::move(w));
    } else {
      per_item.push_back(i);
    }
  }

  if (!fused_geoms.empty()) ITKG_TRY(fused_multi_prepare(fused_geoms, fused_w, &b->fused, &b->plan_lines));
  if (!tile_geoms.empty()) ITKG_TRY(tile2d_multi_prepare(tile_geoms, tile_w, &b->tiles2d, &b->plan_lines));

  // 3. spread the work over kLanes lanes, longest first onto the least loaded
  // lane; the multi-request fused launch counts as one job
  struct Job {
    double work;
    int kind;  // 0 fused multi-request launch, 1 forward item, 2 VJP item, 3 2-D tile class launch
    size_t i;
  };
  std::vector<Job> jobs;
  if (b->fused) {
    double wsum = 0.0;
    for (size_t i = 0; i < b->fwd.size(); ++i)
      if (b->fwd[i].in.dim == 3 && std::find(per_item.begin(), per_item.end(), i) == per_item.end())
        wsum += work_of(b->fwd[i].in, b->fwd[i].requested, b->fwd[i].prm.sigma);
    jobs.push_back({wsum, 0, 0});
  }
  for (int q = 0; q < tile2d_multi_groups(b->tiles2d); ++q) jobs.push_back({tile2d_multi_work(b->tiles2d, q), 3, (size_t)q});
  for (size_t i : per_item) jobs.push_back({work_of(b->fwd[i].in, b->fwd[i].requested, b->fwd[i].prm.sigma), 1, i});
  for (size_t i = 0; i < b->vjp.size(); ++i)
    jobs.push_back({3.0 * work_of(b->vjp[i].x, b->vjp[i].x.region, b->vjp[i].prm.sigma), 2, i});
  std::stable_sort(jobs.begin(), jobs.end(), [](const Job& a, const Job& c) { return a.work > c.work; });
  std::vector<int> lane_of(jobs.size());
  {
    double load[kLanes] = {0.0};
    for (size_t j = 0; j < jobs.size(); ++j) {
      const int l = (int)(std::min_element(load, load + kLanes) - load);
      lane_of[j] = l;
      load[l] += jobs[j].work;
    }
  }

  // 4. capture: lane 0 is the capture stream, the others fork from it and join back
  cudaStream_t lanes[kLanes] = {nullptr};
  cudaEvent_t fork = nullptr, joins[kLanes] = {nullptr};
  itkg_status st = ITKG_SUCCESS;
  for (int l = 0; l < kLanes && st == ITKG_SUCCESS; ++l) {
    st = cuda_status(cudaStreamCreateWithFlags(&lanes[l], cudaStreamNonBlocking), "cudaStreamCreate");
    if (st == ITKG_SUCCESS) st = cuda_status(cudaEventCreateWithFlags(&joins[l], cudaEventDisableTiming), "event");
  }
  if (st == ITKG_SUCCESS) st = cuda_status(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming), "event");
  auto release = [&]() {
    for (int l = 0; l < kLanes; ++l) {
      if (lanes[l]) cudaStreamDestroy(lanes[l]);
      if (joins[l]) cudaEventDestroy(joins[l]);
    }
    if (fork) cudaEventDestroy(fork);
  };
  if (st != ITKG_SUCCESS) {
    release();
    return st;
  }
  cudaStream_t cap = lanes[0];
  const uint64_t launches0 = itkg_launch_counter();
  cudaError_t ce = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
  if (ce != cudaSuccess) {
    release();
    return cuda_status(ce, "cudaStreamBeginCapture");
  }
  st = cuda_status(cudaEventRecord(fork, cap), "cudaEventRecord");
  for (int l = 1; l < kLanes && st == ITKG_SUCCESS; ++l)
    st = cuda_status(cudaStreamWaitEvent(lanes[l], fork, 0), "cudaStreamWaitEvent");
  for (size_t j = 0; j < jobs.size() && st == ITKG_SUCCESS; ++j) {
    cudaStream_t ls = lanes[lane_of[j]];
    const std::string lane = " (lane " + std::to_string(lane_of[j]) + ")";
    if (jobs[j].kind == 0) {
      st = fused_multi_launch(b->fused, ls);
      if (st == ITKG_SUCCESS) b->plan_lines.push_back("fused multi-request launches" + lane);
    } else if (jobs[j].kind == 3) {
      st = tile2d_multi_launch(b->tiles2d, (int)jobs[j].i, ls);
      if (st == ITKG_SUCCESS) b->plan_lines.push_back("2-D tile class " + std::to_string(jobs[j].i) + lane);
    } else if (jobs[j].kind == 1) {
      const size_t i = jobs[j].i;
      itkg_batch::Fwd f = b->fwd[i];
      // items without a multi-request kernel (2-D) still take their single fused kernel
      f.prm.algorithm = (algo[i] == ITKG_ALGO_PER_AXIS || algo[i] == ITKG_ALGO_TWO_PASS) ? algo[i] : ITKG_ALGO_AUTO;
      st = itkg_gaussian_generate_region(&f.in, &f.largest, &f.requested, &f.prm, &f.out, ls);
      b->plan_lines.push_back(std::string("item ") + std::to_string(i) + ": " + itkg_last_kernel() + lane);
    } else {
      itkg_batch::Vjp& v = b->vjp[jobs[j].i];
      st = itkg_gaussian_vjp(&v.x, &v.ybar, &v.prm, v.has_xbar ? &v.xbar : nullptr, v.sigma_bar, v.flags, ls);
      b->plan_lines.push_back(std::string("vjp ") + std::to_string(jobs[j].i) + ": " + itkg_last_kernel() + lane);
    }
  }
  for (int l = 1; l < kLanes; ++l) {
    // join every lane back (also after a failure, so that the capture ends cleanly)
    if (cudaEventRecord(joins[l], lanes[l]) == cudaSuccess) cudaStreamWaitEvent(cap, joins[l], 0);
  }
  cudaGraph_t graph = nullptr;
  ce = cudaStreamEndCapture(cap, &graph);
  release();
  if (st != ITKG_SUCCESS) {
    if (graph) cudaGraphDestroy(graph);
    return st;
  }
  if (ce != cudaSuccess) return cuda_status(ce, "cudaStreamEndCapture");
  b->launches_per_run = itkg_launch_counter() - launches0;
  b->graph = graph;
  ITKG_CUDA(cudaGraphInstantiate(&b->exec, graph, 0));
  return ITKG_SUCCESS;
}

itkg_status itkg_batch_run(itkg_batch* b, void* stream) {
  if (!b || !b->exec) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "batch not planned");
  ITKG_CUDA(cudaGraphLaunch(b->exec, static_cast<cudaStream_t>(stream)));
  note_launches(b->launches_per_run, "batch_graph");
  return ITKG_SUCCESS;
}

const char* itkg_batch_describe(itkg_batch* b) {
  if (!b) return "";
  b->described.clear();
  for (const std::string& l : b->plan_lines) b->described += l + "\n";
  return b->described.c_str();
}

}  // extern "C"
