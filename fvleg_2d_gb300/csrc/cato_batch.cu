// cato_batch.cu -- C-ABI of the batched engine: many independent grid instances of uneven
// sizes advanced together (the batched workload of 256 random-circle grids and the serving stream).
//
// * Every instance has its own state buffers (as a single-instance handle), its own CFL dt, time,
//   iteration count and stop condition (t_end, max_steps), kept in a device descriptor.
// * One step = batch_step_begin (one thread per instance: step decision, dt) + one persistent
//   launch per RK stage and per (flux, reconstruction) group + batch_step_end.  A persistent
//   launch runs as many CTAs as fit on the GPU; each pulls (instance, tile) work items from a
//   device queue, so uneven grids balance dynamically and 256 grids cost the launches of one.
// * Steps run in chunks captured once in a CUDA graph and replayed; the graph is re-captured only
//   when the instance set or the plan changes.
// * Results of an instance do not depend on which other instances share the batch (no cross-
//   instance reduction), so an instance alone and in a mix gives the same state.
#include <algorithm>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/cato_gpu.h"
#include "cato_kernels.cuh"
#include "cato_launch.cuh"
#include "cato_setup.cuh"

using namespace cato;

namespace {

__global__ void batch_step_begin(InstDesc* descs, int n, int* counters, int n_counters) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n_counters) counters[i] = 0;
  if (i >= n) return;
  InstDesc& d = descs[i];
  StepCtl& c = d.ctl;
  if (!d.in_use) {
    c.active = 0;
    return;
  }
  int act = (c.status == 0) && (c.time < c.t_end) && (c.iter < c.max_iter);
  c.active = act;
  if (!act) return;
  double dt = c.fixed_dt > 0.0 ? c.fixed_dt : decode_dt(c.dt_min);
  c.dt = dt;
  c.time = c.time + dt;
  c.iter = c.iter + 1;
  c.dt_min = ~0ULL;
}

// after the last stage: the uploaded primitives have been consumed
__global__ void batch_step_end(InstDesc* descs, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  InstDesc& d = descs[i];
  if (d.in_use && d.ctl.active) d.raw_pending = 0;
}

cudaError_t launch_batch_prec(int prec, int flux, int recon, int threads, cudaStream_t s,
                              const BatchStageArgs& B) {
  if (prec == CATO_FP64) return launch_batch<double>(flux, recon, threads, s, B);
  if (prec == CATO_MIXED_DF) return launch_batch<df>(flux, recon, threads, s, B);
  return launch_batch<float>(flux, recon, threads, s, B);
}

struct StageSpec {
  int kind;
  double a, b, coef;
};

std::vector<StageSpec> stages_of(int rk) {
  std::vector<StageSpec> s;
  if (rk == CATO_RK_SSP2) {
    s.push_back({0, 1.0, 0.0, 1.0});
    s.push_back({1, 0.5, 0.5, 0.5});
  } else if (rk == CATO_RK_SSP3) {
    s.push_back({0, 1.0, 0.0, 1.0});
    s.push_back({1, 3.0 / 4.0, 1.0 / 4.0, 1.0 / 4.0});
    s.push_back({1, 1.0 / 3.0, 2.0 / 3.0, 2.0 / 3.0});
  } else {
    static const double a13[] = {0.1481, 0.4, 1.0}, a14[] = {0.0833, 0.2069, 0.4265, 1.0},
                        a15[] = {0.0533, 0.1263, 0.2375, 0.4414, 1.0},
                        a23[] = {0.1918, 0.4929, 1.0}, a24[] = {0.1084, 0.2602, 0.5052, 1.0},
                        a25[] = {0.0695, 0.1602, 0.2898, 0.5060, 1.0};
    const double* al;
    int ns;
    switch (rk) {
      case CATO_RK_1_3: al = a13; ns = 3; break;
      case CATO_RK_1_4: al = a14; ns = 4; break;
      case CATO_RK_1_5: al = a15; ns = 5; break;
      case CATO_RK_2_3: al = a23; ns = 3; break;
      case CATO_RK_2_4: al = a24; ns = 4; break;
      default: al = a25; ns = 5; break;
    }
    for (int m = 0; m < ns; ++m) s.push_back({0, 1.0, 0.0, al[m]});
  }
  return s;
}

int recon_id(int limiter) {
  return limiter == CATO_LIM_MLP3 ? 3 : (limiter == CATO_LIM_MLP5 ? 5 : 0);
}

struct Group {
  int flux, recon;
  int4* d_items = nullptr;
  int n_items = 0, cap = 0;
};

}  // namespace

struct cato_batch {
  int capacity = 0, prec = 0, rk = 0;
  std::vector<StageSpec> stages;
  cudaStream_t stream = nullptr;
  InstDesc* d_descs = nullptr;
  std::vector<InstDesc> h_descs;
  std::vector<size_t> inst_bytes;
  std::vector<Group> groups;
  int* d_counters = nullptr;
  int n_counters_cap = 0;
  int threads = 128, rows = 32;  // plan: CTA width, largest rows per tile
  int tile_rows = 32;            // rows per tile chosen by the last rebuild
  int sms = 0;
  // one stream per (flux, reconstruction) group: the groups touch disjoint instances, so their
  // stage chains run concurrently between the step's begin and end kernels
  std::vector<cudaStream_t> side;
  std::vector<cudaEvent_t> side_done;
  cudaEvent_t fork = nullptr;
  bool dirty = true;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  int graph_steps = 0;
  InstDesc* h_pinned = nullptr;  // pinned staging for descriptor reads
};

static int bcheck(cudaError_t e) { return e == cudaSuccess ? CATO_OK : CATO_ERR_CUDA; }
#define BK(call)                                   \
  do {                                             \
    cudaError_t _e = (call);                       \
    if (_e != cudaSuccess) {                       \
      (void)cudaGetLastError();                    \
      return CATO_ERR_CUDA;                        \
    }                                              \
  } while (0)

static void free_instance(InstDesc& d) {
  for (int v = 0; v < 4; ++v) {
    cudaFree(d.U[v]);
    for (int s = 0; s < 2; ++s) cudaFree(d.S[s][v]);
  }
  std::memset(&d, 0, sizeof(d));
}

static void drop_graph(cato_batch* b) {
  if (b->graph_exec) cudaGraphExecDestroy(b->graph_exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->graph_exec = nullptr;
  b->graph = nullptr;
  b->graph_steps = 0;
}

// Rebuild the per-group work lists (instance, tile x, tile y), largest instances first so the
// dynamic queue ends on small items.
static int rebuild(cato_batch* b) {
  std::map<std::pair<int, int>, std::vector<int4>> lists;
  std::vector<int> order;
  for (int i = 0; i < b->capacity; ++i)
    if (b->h_descs[i].in_use) order.push_back(i);
  std::sort(order.begin(), order.end(), [&](int x, int y) {
    return (long long)b->h_descs[x].ni * b->h_descs[x].nj >
           (long long)b->h_descs[y].ni * b->h_descs[y].nj;
  });
  if (!b->sms) {
    int dev = 0;
    BK(cudaGetDevice(&dev));
    BK(cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev));
  }
  // Rows per tile: the plan's, halved (down to 4) while the batch would give fewer than two
  // tiles per SM, so that a batch of small grids still fills the GPU.
  auto n_tiles = [&](int r) {
    long long n = 0;
    for (int i : order) {
      const InstDesc& d = b->h_descs[i];
      const int W = b->threads - 2 * d.ng, rr = std::min(r, d.nj);
      n += (long long)((d.ni + W - 1) / W) * ((d.nj + rr - 1) / rr);
    }
    return n;
  };
  int tile_rows = b->rows;
  while (tile_rows > 4 && n_tiles(tile_rows) < 2LL * b->sms) tile_rows = std::max(4, tile_rows / 2);
  b->tile_rows = tile_rows;
  for (int i : order) {
    const InstDesc& d = b->h_descs[i];
    const int W = b->threads - 2 * d.ng;
    const int rows = std::min(tile_rows, d.nj);
    const int tx = (d.ni + W - 1) / W, ty = (d.nj + rows - 1) / rows;
    auto& L = lists[{d.flux, d.recon}];
    for (int y = 0; y < ty; ++y)
      for (int x = 0; x < tx; ++x) L.push_back(make_int4(i, x, y, rows));
  }
  for (auto& g : b->groups) cudaFree(g.d_items);
  b->groups.clear();
  for (auto& kv : lists) {
    Group g;
    g.flux = kv.first.first;
    g.recon = kv.first.second;
    g.n_items = (int)kv.second.size();
    g.cap = g.n_items;
    BK(cudaMalloc(&g.d_items, sizeof(int4) * g.cap));
    BK(cudaMemcpyAsync(g.d_items, kv.second.data(), sizeof(int4) * g.n_items,
                       cudaMemcpyHostToDevice, b->stream));
    b->groups.push_back(g);
  }
  const int need = (int)(b->stages.size() * std::max<size_t>(1, b->groups.size()));
  if (need > b->n_counters_cap) {
    cudaFree(b->d_counters);
    BK(cudaMalloc(&b->d_counters, sizeof(int) * need));
    b->n_counters_cap = need;
  }
  while (b->side.size() < b->groups.size()) {
    cudaStream_t st;
    cudaEvent_t ev;
    BK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    BK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    b->side.push_back(st);
    b->side_done.push_back(ev);
  }
  if (!b->fork) BK(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
  // set each kernel's shared-memory attribute outside any stream capture
  for (const auto& g : b->groups) {
    BatchStageArgs B;
    std::memset(&B, 0, sizeof(B));
    BK(launch_batch_prec(b->prec, g.flux, g.recon, b->threads, b->stream, B));
  }
  BK(cudaStreamSynchronize(b->stream));
  drop_graph(b);
  b->dirty = false;
  return CATO_OK;
}

static int enqueue_batch_step(cato_batch* b) {
  const int nb = (std::max(b->capacity, b->n_counters_cap) + 127) / 128;
  batch_step_begin<<<nb, 128, 0, b->stream>>>(b->d_descs, b->capacity, b->d_counters,
                                              b->n_counters_cap);
  BK(cudaGetLastError());
  const int ns = (int)b->stages.size();
  const int ng = (int)b->groups.size();
  const bool fan = ng > 1;
  if (fan) BK(cudaEventRecord(b->fork, b->stream));
  for (int g = 0; g < ng; ++g) {
    const Group& G = b->groups[g];
    cudaStream_t st = fan ? b->side[g] : b->stream;
    if (fan) BK(cudaStreamWaitEvent(st, b->fork, 0));
    for (int k = 0; k < ns; ++k) {
      BatchStageArgs B;
      B.descs = b->d_descs;
      B.items = G.d_items;
      B.n_items = G.n_items;
      B.counter = b->d_counters + k * ng + g;
      B.stage = k;
      B.kind = b->stages[k].kind;
      B.last = (k == ns - 1);
      B.a = b->stages[k].a;
      B.b = b->stages[k].b;
      B.coef = b->stages[k].coef;
      BK(launch_batch_prec(b->prec, G.flux, G.recon, b->threads, st, B));
    }
    if (fan) {
      BK(cudaEventRecord(b->side_done[g], st));
      BK(cudaStreamWaitEvent(b->stream, b->side_done[g], 0));
    }
  }
  batch_step_end<<<(b->capacity + 127) / 128, 128, 0, b->stream>>>(b->d_descs, b->capacity);
  BK(cudaGetLastError());
  return CATO_OK;
}

extern "C" {

int cato_batch_instance_bytes(const cato_config* cfg, uint64_t* bytes) {
  if (!cfg || !bytes) return CATO_ERR_ARG;
  const size_t pitch = (size_t)(cfg->ni + 31) / 32 * 32;
  const size_t cells = pitch * (size_t)cfg->nj;
  // every precision: U + two stage buffers of four FP64 fields
  *bytes = cells * 8 * 12;
  return CATO_OK;
}

int cato_batch_create(int32_t capacity, int32_t precision, int32_t rk, cato_batch** out) {
  if (!out || capacity < 1) return CATO_ERR_ARG;
  if (precision != CATO_FP64 && precision != CATO_MIXED && precision != CATO_MIXED_DF)
    return CATO_ERR_CONFIG;
  if (rk < CATO_RK_SSP2 || rk > CATO_RK_2_5) return CATO_ERR_CONFIG;
  *out = nullptr;
  cato_batch* b = new cato_batch();
  b->capacity = capacity;
  b->prec = precision;
  b->rk = rk;
  b->stages = stages_of(rk);
  b->h_descs.assign(capacity, InstDesc{});
  for (auto& d : b->h_descs) std::memset(&d, 0, sizeof(d));
  b->inst_bytes.assign(capacity, 0);
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMalloc(&b->d_descs, sizeof(InstDesc) * capacity) != cudaSuccess ||
      cudaMallocHost(&b->h_pinned, sizeof(InstDesc) * capacity) != cudaSuccess) {
    (void)cudaGetLastError();
    cato_batch_destroy(b);
    return CATO_ERR_OOM;
  }
  if (cudaMemcpy(b->d_descs, b->h_descs.data(), sizeof(InstDesc) * capacity,
                 cudaMemcpyHostToDevice) != cudaSuccess) {
    cato_batch_destroy(b);
    return CATO_ERR_CUDA;
  }
  *out = b;
  return CATO_OK;
}

int cato_batch_destroy(cato_batch* b) {
  if (!b) return CATO_ERR_ARG;
  if (b->stream) cudaStreamSynchronize(b->stream);
  drop_graph(b);
  for (auto& d : b->h_descs)
    if (d.in_use) free_instance(d);
  for (auto& g : b->groups) cudaFree(g.d_items);
  for (size_t k = 0; k < b->side.size(); ++k) {
    cudaStreamDestroy(b->side[k]);
    cudaEventDestroy(b->side_done[k]);
  }
  if (b->fork) cudaEventDestroy(b->fork);
  cudaFree(b->d_counters);
  cudaFree(b->d_descs);
  if (b->h_pinned) cudaFreeHost(b->h_pinned);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return CATO_OK;
}

int cato_batch_set_plan(cato_batch* b, int32_t threads, int32_t rows_per_cta) {
  if (!b || threads < 64 || threads > 256 || threads % 32 || rows_per_cta < 1) return CATO_ERR_ARG;
  b->threads = threads;
  b->rows = rows_per_cta;
  b->dirty = true;
  return CATO_OK;
}

int cato_batch_add(cato_batch* b, const cato_config* cfg, const double* rho, const double* u,
                   const double* v, const double* p, int64_t ld, double t_end, int64_t max_steps,
                   int32_t* slot) {
  if (!b || !cfg || !rho || !u || !v || !p || !slot) return CATO_ERR_ARG;
  int rc = cato_config_check(cfg);
  if (rc != CATO_OK) return rc;
  if (cfg->precision != b->prec || cfg->rk != b->rk) return CATO_ERR_CONFIG;
  // the pressure-input boundary runs per-stage kernels of its own: single handles only
  if (cfg->bc[CATO_PLUS_X] == CATO_BC_PRESSURE_INPUT) return CATO_ERR_CONFIG;
  // slabs of a split grid step through single handles (their ghost rows are exchanged)
  if (cfg->bc[CATO_PLUS_Y] == CATO_BC_EXCHANGE || cfg->bc[CATO_MINUS_Y] == CATO_BC_EXCHANGE)
    return CATO_ERR_CONFIG;
  if (ld < cfg->ni + 2 * cfg->n_ghost) return CATO_ERR_ARG;
  int s = -1;
  for (int i = 0; i < b->capacity; ++i)
    if (!b->h_descs[i].in_use) { s = i; break; }
  if (s < 0) return CATO_ERR_CAPACITY;
  BK(cudaStreamSynchronize(b->stream));
  InstDesc d;
  std::memset(&d, 0, sizeof(d));
  d.ni = cfg->ni;
  d.nj = cfg->nj;
  d.ng = cfg->n_ghost;
  d.pitch = (cfg->ni + 31) / 32 * 32;
  for (int k = 0; k < 4; ++k) d.bc[k] = cfg->bc[k];
  d.limiter = cfg->limiter;
  d.flux = cfg->flux;
  d.recon = recon_id(cfg->limiter);
  d.prec = cfg->precision;
  d.gamma = cfg->gamma;
  d.bc_p = cfg->bc_pressure;
  d.cfl = cfg->cfl;
  // the same constants and uniform geometry as a single-instance handle
  d.K64 = flux_consts_of(*cfg);
  d.K32 = convert_consts<float>(d.K64);
  d.Kdf = convert_consts<df>(d.K64);
  d.G = uniform_geom(cfg->dx, cfg->dy);
  const size_t cells = (size_t)d.pitch * d.nj, fb = cells * sizeof(double);
  bool ok = true;
  for (int k = 0; k < 4 && ok; ++k) {
    ok = cudaMalloc(&d.U[k], fb) == cudaSuccess && cudaMalloc(&d.S[0][k], fb) == cudaSuccess &&
         cudaMalloc(&d.S[1][k], fb) == cudaSuccess;
    d.prim_raw[k] = d.S[1][k];  // S1 is first written by stage 2, after stage 1 read these
  }
  if (!ok) {
    (void)cudaGetLastError();
    free_instance(d);
    return CATO_ERR_OOM;
  }
  const double* src[4] = {rho, u, v, p};
  for (int k = 0; k < 4; ++k)
    BK(cudaMemcpy2DAsync(d.prim_raw[k], (size_t)d.pitch * sizeof(double),
                         src[k] + (size_t)d.ng * ld + d.ng, (size_t)ld * sizeof(double),
                         (size_t)d.ni * sizeof(double), (size_t)d.nj, cudaMemcpyHostToDevice,
                         b->stream));
  d.ctl.dt_min = ~0ULL;
  d.ctl.t_end = t_end;
  d.ctl.max_iter = max_steps >= 0 ? max_steps : (1LL << 62);
  d.raw_pending = 1;
  d.in_use = 1;
  b->h_descs[s] = d;
  BK(cudaMemcpyAsync(b->d_descs + s, &b->h_descs[s], sizeof(InstDesc), cudaMemcpyHostToDevice,
                     b->stream));
  long long n = (long long)d.ni * d.nj;
  int blocks = (int)std::min<long long>((n + 255) / 256, 152LL * 32);
  upload_init_kernel<<<blocks, 256, 0, b->stream>>>(
      d.ni, d.nj, d.pitch, d.gamma, d.cfl, d.G.dx, d.G.dy, nullptr, nullptr, d.prim_raw[0],
      d.prim_raw[1],
      d.prim_raw[2], d.prim_raw[3], d.U[0], d.U[1], d.U[2], d.U[3],
      &b->d_descs[s].ctl);
  BK(cudaGetLastError());
  BK(cudaStreamSynchronize(b->stream));
  uint64_t bytes = 0;
  cato_batch_instance_bytes(cfg, &bytes);
  b->inst_bytes[s] = bytes;
  b->dirty = true;
  *slot = s;
  return CATO_OK;
}

int cato_batch_remove(cato_batch* b, int32_t slot) {
  if (!b || slot < 0 || slot >= b->capacity || !b->h_descs[slot].in_use) return CATO_ERR_ARG;
  BK(cudaStreamSynchronize(b->stream));
  free_instance(b->h_descs[slot]);
  b->inst_bytes[slot] = 0;
  BK(cudaMemcpyAsync(b->d_descs + slot, &b->h_descs[slot], sizeof(InstDesc),
                     cudaMemcpyHostToDevice, b->stream));
  BK(cudaStreamSynchronize(b->stream));
  b->dirty = true;
  return CATO_OK;
}

int cato_batch_step(cato_batch* b, int32_t n_steps, int32_t use_graph, float* device_ms) {
  if (!b || n_steps < 0) return CATO_ERR_ARG;
  int rc;
  if (b->dirty && (rc = rebuild(b))) return rc;
  cudaEvent_t e0, e1;
  BK(cudaEventCreate(&e0));
  BK(cudaEventCreate(&e1));
  BK(cudaEventRecord(e0, b->stream));
  int done = 0;
  const int chunk = 16;
  if (use_graph && n_steps >= chunk) {
    if (!b->graph_exec || b->graph_steps != chunk) {
      drop_graph(b);
      BK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
      for (int s = 0; s < chunk; ++s) {
        rc = enqueue_batch_step(b);
        if (rc) {
          cudaGraph_t tmp;
          cudaStreamEndCapture(b->stream, &tmp);
          if (tmp) cudaGraphDestroy(tmp);
          return rc;
        }
      }
      BK(cudaStreamEndCapture(b->stream, &b->graph));
      BK(cudaGraphInstantiate(&b->graph_exec, b->graph, 0));
      b->graph_steps = chunk;
    }
    for (; done + chunk <= n_steps; done += chunk) BK(cudaGraphLaunch(b->graph_exec, b->stream));
  }
  for (; done < n_steps; ++done)
    if ((rc = enqueue_batch_step(b))) return rc;
  BK(cudaEventRecord(e1, b->stream));
  BK(cudaEventSynchronize(e1));
  float ms = 0.f;
  BK(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (device_ms) *device_ms = ms;
  return CATO_OK;
}

int cato_batch_query(cato_batch* b, int32_t slot, int64_t* iteration, double* time, double* dt,
                     int32_t* running, int32_t* error_code) {
  if (!b || slot < 0 || slot >= b->capacity || !b->h_descs[slot].in_use) return CATO_ERR_ARG;
  BK(cudaMemcpyAsync(b->h_pinned + slot, b->d_descs + slot, sizeof(InstDesc),
                     cudaMemcpyDeviceToHost, b->stream));
  BK(cudaStreamSynchronize(b->stream));
  const InstDesc& d = b->h_pinned[slot];
  if (iteration) *iteration = d.ctl.iter;
  if (time) *time = d.ctl.time;
  if (dt) *dt = d.ctl.dt;
  if (running)
    *running = (d.ctl.status == 0 && d.ctl.time < d.ctl.t_end && d.ctl.iter < d.ctl.max_iter);
  if (error_code) {
    const int bits = d.ctl.status;
    // the reference's order: NaN checks at every stage assignment, then negative density,
    // then negative pressure (mod_fluid.f90:718-737)
    *error_code = (bits & ST_NAN) ? CATO_NANS_FOUND
                  : (bits & ST_NEG_DENSITY) ? CATO_NEG_DENSITY
                  : (bits & ST_NEG_PRESSURE) ? CATO_NEG_PRESSURE : CATO_OK;
  }
  return CATO_OK;
}

int cato_batch_running(cato_batch* b, int32_t* n_running, int32_t* running_flags) {
  if (!b || !n_running) return CATO_ERR_ARG;
  BK(cudaMemcpyAsync(b->h_pinned, b->d_descs, sizeof(InstDesc) * b->capacity,
                     cudaMemcpyDeviceToHost, b->stream));
  BK(cudaStreamSynchronize(b->stream));
  int n = 0;
  for (int i = 0; i < b->capacity; ++i) {
    const InstDesc& d = b->h_pinned[i];
    const int r = d.in_use && d.ctl.status == 0 && d.ctl.time < d.ctl.t_end &&
                  d.ctl.iter < d.ctl.max_iter;
    if (running_flags) running_flags[i] = r;
    n += r;
  }
  *n_running = n;
  return CATO_OK;
}

int cato_batch_download(cato_batch* b, int32_t slot, double* rho, double* rho_u, double* rho_v,
                        double* rho_E, int64_t ld) {
  if (!b || slot < 0 || slot >= b->capacity || !b->h_descs[slot].in_use) return CATO_ERR_ARG;
  BK(cudaMemcpyAsync(b->h_pinned + slot, b->d_descs + slot, sizeof(InstDesc),
                     cudaMemcpyDeviceToHost, b->stream));
  BK(cudaStreamSynchronize(b->stream));
  const InstDesc& d = b->h_pinned[slot];
  if (ld < d.ni + 2 * d.ng) return CATO_ERR_ARG;
  double* const* U = d.U;
  double* out[4] = {rho, rho_u, rho_v, rho_E};
  for (int k = 0; k < 4; ++k) {
    if (!out[k]) continue;
    for (int j = 0; j < d.nj + 2 * d.ng; ++j)
      std::memset(out[k] + (size_t)j * ld, 0, sizeof(double) * (size_t)(d.ni + 2 * d.ng));
    BK(cudaMemcpy2DAsync(out[k] + (size_t)d.ng * ld + d.ng, (size_t)ld * sizeof(double), U[k],
                         (size_t)d.pitch * sizeof(double), (size_t)d.ni * sizeof(double),
                         (size_t)d.nj, cudaMemcpyDeviceToHost, b->stream));
  }
  BK(cudaStreamSynchronize(b->stream));
  return CATO_OK;
}

}  // extern "C"
