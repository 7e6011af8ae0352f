// omhd_ensemble.cu -- ensembles of independent 2D problems advanced together:
// one persistent batched kernel per RK stage for all members, a per-member
// dt / step record / error word, CUDA-graph replay, and an autotuner that
// picks the tile shape and CTAs per SM from measured step times.
#include <cstdio>
#include <cstring>
#include <vector>

#include "omhd_common.cuh"
#include "omhd_fused.h"
#include "omhd_solver_impl.h"
#include "omhd_step.cuh"

using namespace omhd;

struct omhd_ensemble {
  int n = 0;
  int precision = OMHD_PREC_MIXED;
  int flux = OMHD_FLUX_HLLD;
  std::vector<omhd_solver*> members;
  double* pool = nullptr;  // U and U1 of every member
  StageArgs* args_dev[2] = {nullptr, nullptr};
  int* tile_start_dev = nullptr;
  int total_tiles = 0;
  int tile_kind = 0;
  int ctas_per_sm = 1;
  int sms = 152;
  cudaStream_t stream = nullptr;
  cudaGraphExec_t graph = nullptr;
  int graph_steps = 0;
};

namespace {

int ecuda(cudaError_t e) { return e == cudaSuccess ? OMHD_OK : OMHD_CUDA_ERR; }

void drop_graph(omhd_ensemble* e) {
  if (e->graph) cudaGraphExecDestroy(e->graph);
  e->graph = nullptr;
  e->graph_steps = 0;
}

// tile prefix sums for the current tile shape
int build_tiles(omhd_ensemble* e) {
  int tx, ty;
  batch_tile_dims(e->tile_kind, &tx, &ty);
  std::vector<int> ts(e->n + 1, 0);
  for (int i = 0; i < e->n; ++i) {
    const omhd_config& c = e->members[i]->cfg;
    ts[i + 1] = ts[i] + ((c.ix - 2 + tx - 1) / tx) * ((c.jx - 2 + ty - 1) / ty);
  }
  e->total_tiles = ts[e->n];
  return ecuda(cudaMemcpy(e->tile_start_dev, ts.data(), sizeof(int) * (e->n + 1), cudaMemcpyHostToDevice));
}

int upload_args(omhd_ensemble* e) {
  for (int stage = 1; stage <= 2; ++stage) {
    std::vector<StageArgs> h(e->n);
    for (int i = 0; i < e->n; ++i) h[i] = make_stage_args(e->members[i], stage);
    int r = ecuda(cudaMemcpy(e->args_dev[stage - 1], h.data(), sizeof(StageArgs) * e->n, cudaMemcpyHostToDevice));
    if (r) return r;
  }
  return OMHD_OK;
}

int launch_stage(omhd_ensemble* e, int stage) {
  int ctas = e->ctas_per_sm * e->sms;
  if (ctas > e->total_tiles) ctas = e->total_tiles;
  if (ctas < 1) return OMHD_OK;
  const int r = (e->precision == OMHD_PREC_MIXED)
                    ? launch_batch2d_mixed(e->flux, e->tile_kind, e->args_dev[stage - 1], e->tile_start_dev, e->n,
                                           e->total_tiles, ctas, e->stream)
                    : launch_batch2d_fp64(e->flux, e->tile_kind, e->args_dev[stage - 1], e->tile_start_dev, e->n,
                                          e->total_tiles, ctas, e->stream);
  return r ? OMHD_CUDA_ERR : OMHD_OK;
}

}  // namespace

extern "C" {

int omhd_ensemble_destroy(omhd_ensemble* e) {
  if (!e) return OMHD_OK;
  drop_graph(e);
  for (auto* m : e->members) omhd_solver_destroy(m);
  cudaFree(e->pool);
  cudaFree(e->args_dev[0]);
  cudaFree(e->args_dev[1]);
  cudaFree(e->tile_start_dev);
  delete e;
  return OMHD_OK;
}

int omhd_ensemble_create(const omhd_config* cfgs, int n, omhd_ensemble** out) {
  if (!cfgs || n <= 0 || !out) return OMHD_BAD_ARG;
  *out = nullptr;
  const int prec = cfgs[0].precision, flux = cfgs[0].flux_type;
  if (prec != OMHD_PREC_MIXED && prec != OMHD_PREC_FP64) return OMHD_NOT_SUPPORTED;
  if (flux != OMHD_FLUX_HLLD) return OMHD_NOT_SUPPORTED;
  for (int i = 0; i < n; ++i)
    if (cfgs[i].nd != 2 || cfgs[i].precision != prec || cfgs[i].flux_type != flux) return OMHD_NOT_SUPPORTED;
  for (int i = 0; i < n; ++i) {  // every member is checked before anything is allocated
    const int v = validate_config(&cfgs[i]);
    if (v) return v;
  }
  omhd_ensemble* e = new omhd_ensemble();
  e->n = n;
  e->precision = prec;
  e->flux = flux;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&e->sms, cudaDevAttrMultiProcessorCount, dev);
  size_t total = 0;
  for (int i = 0; i < n; ++i) total += 2 * (size_t)NV * cfgs[i].ix * cfgs[i].jx;
  int r = ecuda(cudaMalloc(&e->pool, sizeof(double) * total));
  size_t off = 0;
  for (int i = 0; i < n && !r; ++i) {
    omhd_solver* s = nullptr;
    r = omhd_solver_create(&cfgs[i], &s);
    if (r) break;
    e->members.push_back(s);
    const size_t ni = (size_t)NV * cfgs[i].ix * cfgs[i].jx;
    r = omhd_solver_bind(s, e->pool + off, e->pool + off + ni);
    off += 2 * ni;
  }
  if (!r) r = ecuda(cudaMalloc(&e->args_dev[0], sizeof(StageArgs) * n));
  if (!r) r = ecuda(cudaMalloc(&e->args_dev[1], sizeof(StageArgs) * n));
  if (!r) r = ecuda(cudaMalloc(&e->tile_start_dev, sizeof(int) * (n + 2)));  // prefix sums + work counter
  if (!r) r = upload_args(e);
  if (!r) r = build_tiles(e);
  if (r) {
    omhd_ensemble_destroy(e);
    return r;
  }
  *out = e;
  return OMHD_OK;
}

int omhd_ensemble_size(omhd_ensemble* e) { return e ? e->n : 0; }

int omhd_ensemble_set_stream(omhd_ensemble* e, void* stream) {
  if (!e) return OMHD_BAD_ARG;
  drop_graph(e);
  e->stream = (cudaStream_t)stream;
  for (auto* m : e->members) omhd_solver_set_stream(m, stream);
  return OMHD_OK;
}

int omhd_ensemble_member(omhd_ensemble* e, int i, omhd_solver** s) {
  if (!e || !s || i < 0 || i >= e->n) return OMHD_BAD_ARG;
  *s = e->members[i];
  return OMHD_OK;
}

int omhd_ensemble_init_models(omhd_ensemble* e, const omhd_model* models) {
  if (!e || !models) return OMHD_BAD_ARG;
  for (int i = 0; i < e->n; ++i) {
    const int r = omhd_solver_init_model(e->members[i], &models[i]);
    if (r) return r;
  }
  return OMHD_OK;
}

int omhd_ensemble_set_tiling(omhd_ensemble* e, int tile_kind, int ctas_per_sm) {
  if (!e || tile_kind < 0 || tile_kind >= kBatchTileKinds || ctas_per_sm < 1 || ctas_per_sm > 8) return OMHD_BAD_ARG;
  drop_graph(e);
  e->tile_kind = tile_kind;
  e->ctas_per_sm = ctas_per_sm;
  return build_tiles(e);
}

int omhd_ensemble_step(omhd_ensemble* e, int nsteps) {
  if (!e || nsteps < 0) return OMHD_BAD_ARG;
  for (int k = 0; k < nsteps; ++k) {
    int r = launch_stage(e, 1);
    if (r) return r;
    r = launch_stage(e, 2);
    if (r) return r;
  }
  return OMHD_OK;
}

int omhd_ensemble_step_graph(omhd_ensemble* e, int nsteps, int replays) {
  if (!e || nsteps <= 0 || replays < 0) return OMHD_BAD_ARG;
  if (!e->stream) return OMHD_NOT_SUPPORTED;
  if (e->graph_steps != nsteps) {
    drop_graph(e);
    cudaGraph_t g;
    if (cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return OMHD_CUDA_ERR;
    const int lr = omhd_ensemble_step(e, nsteps);
    const cudaError_t ce = cudaStreamEndCapture(e->stream, &g);
    if (lr) return lr;
    if (ce != cudaSuccess) return OMHD_CUDA_ERR;
    const cudaError_t ie = cudaGraphInstantiate(&e->graph, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) return OMHD_CUDA_ERR;
    e->graph_steps = nsteps;
  }
  for (int q = 0; q < replays; ++q)
    if (cudaGraphLaunch(e->graph, e->stream) != cudaSuccess) return OMHD_CUDA_ERR;
  return OMHD_OK;
}

// Measures `steps` real steps with every tile shape and CTAs-per-SM choice
// (tiling does not change the arithmetic of any cell, so the steps taken while
// tuning are ordinary steps of the run) and keeps the fastest.
int omhd_ensemble_autotune(omhd_ensemble* e, int steps, int* best_kind, int* best_ctas, double* best_ms) {
  if (!e || steps <= 0) return OMHD_BAD_ARG;
  // every candidate is timed from the same ensemble state: the states, step
  // records and error words are saved here and put back before each
  // measurement and at the end, so tuning leaves the ensemble where it was
  size_t pool_doubles = 0;
  for (int i = 0; i < e->n; ++i) pool_doubles += 2 * e->members[i]->n * NV;
  double* snap = nullptr;
  std::vector<StepState> st_h(e->n);
  std::vector<DevError> er_h(e->n);
  if (cudaStreamSynchronize(e->stream) != cudaSuccess) return OMHD_CUDA_ERR;
  if (cudaMalloc(&snap, sizeof(double) * pool_doubles) != cudaSuccess) return OMHD_CUDA_ERR;
  int rs = ecuda(cudaMemcpy(snap, e->pool, sizeof(double) * pool_doubles, cudaMemcpyDeviceToDevice));
  for (int i = 0; i < e->n && !rs; ++i) {
    rs = ecuda(cudaMemcpy(&st_h[i], e->members[i]->st, sizeof(StepState), cudaMemcpyDeviceToHost));
    if (!rs) rs = ecuda(cudaMemcpy(&er_h[i], e->members[i]->err, sizeof(DevError), cudaMemcpyDeviceToHost));
  }
  auto restore = [&]() -> int {
    if (cudaStreamSynchronize(e->stream) != cudaSuccess) return OMHD_CUDA_ERR;
    int r = ecuda(cudaMemcpy(e->pool, snap, sizeof(double) * pool_doubles, cudaMemcpyDeviceToDevice));
    for (int i = 0; i < e->n && !r; ++i) {
      r = ecuda(cudaMemcpy(e->members[i]->st, &st_h[i], sizeof(StepState), cudaMemcpyHostToDevice));
      if (!r) r = ecuda(cudaMemcpy(e->members[i]->err, &er_h[i], sizeof(DevError), cudaMemcpyHostToDevice));
    }
    return r;
  };
  if (rs) {
    cudaFree(snap);
    return rs;
  }
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  double best = 1e300;
  int bk = 0, bc = 1;
  for (int kind = 0; kind < kBatchTileKinds; ++kind)
    for (int cps = 1; cps <= batch_max_ctas(kind, e->precision == OMHD_PREC_MIXED); ++cps) {
      int r = omhd_ensemble_set_tiling(e, kind, cps);
      if (r) continue;
      r = omhd_ensemble_step(e, 1);  // warm-up: first launch configures the kernel
      if (r) continue;
      if (restore()) break;
      cudaEventRecord(a, e->stream);
      r = omhd_ensemble_step(e, steps);
      cudaEventRecord(b, e->stream);
      if (cudaEventSynchronize(b) != cudaSuccess || r) continue;
      float ms = 0;
      cudaEventElapsedTime(&ms, a, b);
      if (ms / steps < best) {
        best = ms / steps;
        bk = kind;
        bc = cps;
      }
    }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaGetLastError();
  const int rr = restore();
  cudaFree(snap);
  if (rr) return rr;
  if (best_kind) *best_kind = bk;
  if (best_ctas) *best_ctas = bc;
  if (best_ms) *best_ms = best;
  return omhd_ensemble_set_tiling(e, bk, bc);
}

int omhd_ensemble_sync(omhd_ensemble* e, omhd_step_info* infos) {
  if (!e) return OMHD_BAD_ARG;
  if (cudaStreamSynchronize(e->stream) != cudaSuccess) return OMHD_CUDA_ERR;
  int first = OMHD_OK;
  for (int i = 0; i < e->n; ++i) {
    omhd_step_info inf;
    const int r = omhd_solver_sync(e->members[i], &inf);
    if (infos) infos[i] = inf;
    if (r && !first) first = r;
  }
  return first;
}

}  // extern "C"
