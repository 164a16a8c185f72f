// Batched hopping term: many independent instances (each with its own lattice volume, Ls,
// right-hand sides, gauge field and storage precision FP32 or FP16) applied in ONE
// persistent launch that is captured once in a CUDA graph and replayed.
//
// Work decomposition.  A thread owns `spt` consecutive innermost slices (e = s*nrhs + rhs)
// of one site; the slices of a site are cut into `split` contiguous tiles of TE = LsE/split
// slices, so a tile holds TE/nrhs values of s with all right-hand sides (an Ls tile) or, when
// TE < nrhs, TE of the right-hand sides at one s (an RHS tile).  Threads are ordered (tile,
// site, slice group), and an instance's threads are cut into work items of one warp each.  The
// link of a (site, leg) is loaded once per thread group and reused over its tile's slices;
// more tiles put more sites in a CTA.
//
// Scheduling.  A grid of (SMs x resident CTAs per SM) CTAs pulls items from a device counter,
// warp by warp; each warp claims its next item while it works on the current one, so the
// atomic's latency is hidden and uneven volumes still balance dynamically.  Items run largest
// instance first.
// The loop is bounded by the item count and never waits on another CTA.  A memset node in the
// same graph resets the counter.
//
// Kernels.  Rows of 8, 12, 16, 24, 32, 48 or 64 slots (Ls = 8/12/16 with 1, 2 or 4 right-hand
// sides) take a path with the row stride a compile-time constant, as the single-instance
// specialised form does; other extents, and BF16 links, take the runtime-stride path.  Registers are capped so that (threads x CTAs per SM)
// ~ 384 threads stay resident, the operating point of the single-instance kernels.
//
// Tuning.  The shape (threads per CTA, slices per thread for FP32 and FP16 instances, tile
// split) is chosen by timing graph replays of the caller's own batch.
#include <algorithm>
#include <vector>

#include "common.cuh"
#include "dhop_kernel.cuh"

namespace gbdw {
namespace {

struct BatchInst {
  DhopParams p;
  unsigned nthreads;      // nsite * LsE / spt
  unsigned tile_threads;  // nsite * TE / spt (threads of one tile)
  int kind;               // 0: F32/F32, 1: F16/F16-gauge, 2: F16/BF16-gauge
  int spt;
  int TE;                 // slices per tile
  int lsp;                // compile-time row stride path: 8, 12, 16 or 0 (runtime)
};

// One thread of an instance: tile, site and first slice from the thread index.
template <int PIN, int GP, int DAG, int N, int LSPC>
__device__ __forceinline__ void batch_thread(const BatchInst& I, unsigned tid) {
  DhopParams p = I.p;
  if constexpr (LSPC > 0) {
    p.LsE = LSPC;
    p.LsP = LSPC;
  }
  const unsigned tile = tid / I.tile_threads;
  const unsigned r = tid - tile * I.tile_threads;
  const unsigned G = unsigned(I.TE) / N;
  const unsigned site = r / G;
  const int s0 = int(tile) * I.TE + int(r - site * G) * N;
  using T = typename Arith<PIN>::T;
  cpx<T> acc[N][12];
  dhop_thread<PIN, GP, DAG, N>(p, site, s0, acc);
  store_spinor<PIN, N>(p.out, p.out_norm, site, s0, p.LsE, p.LsP, acc);
}

template <int PIN, int GP, int DAG, int N>
__device__ __forceinline__ void batch_by_rows(const BatchInst& I, unsigned tid) {
  if constexpr (GP == GBDW_BF16) {
    batch_thread<PIN, GP, DAG, N, 0>(I, tid);
  } else {
    switch (I.lsp) {
      case 8: batch_thread<PIN, GP, DAG, N, 8>(I, tid); break;
      case 12: batch_thread<PIN, GP, DAG, N, 12>(I, tid); break;
      case 16: batch_thread<PIN, GP, DAG, N, 16>(I, tid); break;
      case 24: batch_thread<PIN, GP, DAG, N, 24>(I, tid); break;
      case 32: batch_thread<PIN, GP, DAG, N, 32>(I, tid); break;
      case 48: batch_thread<PIN, GP, DAG, N, 48>(I, tid); break;
      case 64: batch_thread<PIN, GP, DAG, N, 64>(I, tid); break;
      default: batch_thread<PIN, GP, DAG, N, 0>(I, tid); break;
    }
  }
}

template <int PIN, int GP, int DAG>
__device__ __forceinline__ void batch_by_spt(const BatchInst& I, unsigned tid) {
  if (I.spt == 2) batch_by_rows<PIN, GP, DAG, 2>(I, tid);
  else batch_thread<PIN, GP, DAG, 1, 0>(I, tid);
}

// Work items are one warp each; every warp claims its own items (lane 0 takes the next one
// from the counter while the warp works on the current one), so the warps of a CTA never wait
// for each other.
template <int DAG, int T, int MINB>
__global__ void __launch_bounds__(T, MINB) k_batch(const BatchInst* __restrict__ inst,
                                                   const unsigned short* __restrict__ item_inst,
                                                   const unsigned* __restrict__ item_begin, unsigned total,
                                                   unsigned* next) {
  const unsigned lane = threadIdx.x & 31u;
  unsigned cur = 0, nxt = 0;
  if (lane == 0) {
    cur = atomicAdd(next, 1u);
    nxt = atomicAdd(next, 1u);
  }
  cur = __shfl_sync(0xffffffffu, cur, 0);
  nxt = __shfl_sync(0xffffffffu, nxt, 0);
  // claims only grow, so once the current item is past the end the queued one is too
  while (cur < total) {
    unsigned claim = 0;
    if (lane == 0) claim = atomicAdd(next, 1u);  // latency hidden behind the work below
    const int k = item_inst[cur];
    const BatchInst& I = inst[k];
    const unsigned tid = (cur - item_begin[k]) * 32u + lane;
    if (tid < I.nthreads) {
      if (I.kind == 0) batch_by_spt<GBDW_F32, GBDW_F32, DAG>(I, tid);
      else if (I.kind == 1) batch_by_spt<GBDW_F16, GBDW_F16, DAG>(I, tid);
      else batch_by_spt<GBDW_F16, GBDW_BF16, DAG>(I, tid);
    }
    cur = nxt;
    nxt = __shfl_sync(0xffffffffu, claim, 0);
  }
}

}  // namespace
}  // namespace gbdw

using namespace gbdw;

struct gbdw_batch {
  std::vector<const gbdw_gauge*> g;
  std::vector<gbdw_field*> out;
  std::vector<const gbdw_field*> in;
  int dag = 0;
  int threads = 128;
  int spt32 = 2, spt16 = 2;
  int split = 1;
  BatchInst* d_inst = nullptr;
  unsigned* d_next = nullptr;
  unsigned* d_begin = nullptr;
  unsigned short* d_item_inst = nullptr;
  size_t item_cap = 0;
  unsigned total = 0;
  int grid = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

namespace {

int kind_of(const gbdw_gauge* g, const gbdw_field* f) {
  if (f->prec == GBDW_F32 && g->prec == GBDW_F32) return 0;
  if (f->prec == GBDW_F16 && g->prec == GBDW_F16) return 1;
  if (f->prec == GBDW_F16 && g->prec == GBDW_BF16) return 2;
  return -1;
}

void release_graph(gbdw_batch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
}

template <int DAG, int T, int MINB>
cudaError_t occupancy_of(int* per_sm) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k_batch<DAG, T, MINB>, T, 0);
}

template <int DAG>
cudaError_t occupancy(int threads, int* per_sm) {
  if (threads == 64) return occupancy_of<DAG, 64, 6>(per_sm);
  return occupancy_of<DAG, 128, 3>(per_sm);
}

template <int DAG>
void launch(const gbdw_batch* b, cudaStream_t s) {
  if (b->threads == 64)
    k_batch<DAG, 64, 6><<<b->grid, 64, 0, s>>>(b->d_inst, b->d_item_inst, b->d_begin, b->total, b->d_next);
  else
    k_batch<DAG, 128, 3><<<b->grid, 128, 0, s>>>(b->d_inst, b->d_item_inst, b->d_begin, b->total, b->d_next);
}

// Tile of an instance for the batch's split: the largest split <= the batch's that cuts the
// extent into whole slice groups and whose tile is whole values of s (a multiple of nrhs) or
// whole sets of right-hand sides at one s (a divisor of nrhs).
int tile_of(int LsE, int nrhs, int spt, int split) {
  for (int sp = split; sp > 1; sp >>= 1) {
    if (LsE % sp) continue;
    const int TE = LsE / sp;
    if (TE % spt == 0 && (TE % nrhs == 0 || nrhs % TE == 0)) return TE;
  }
  return LsE;
}

// Builds the work list for the current shape and captures [reset counter, persistent kernel].
int build(gbdw_batch* b) {
  release_graph(b);
  const int n = int(b->g.size());
  std::vector<BatchInst> hi(n);
  std::vector<unsigned> begin(n);
  // largest instances first so the tail of the dynamic schedule is made of small items
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int c) {
    return b->in[a]->lat->nsite * b->in[a]->LsE > b->in[c]->lat->nsite * b->in[c]->LsE;
  });
  unsigned items = 0;
  std::vector<unsigned short> item_inst;
  for (int k = 0; k < n; ++k) {
    const int i = order[k];
    BatchInst& I = hi[k];
    gbdw_field* o = b->out[i];
    const gbdw_field* x = b->in[i];
    const gbdw_gauge* g = b->g[i];
    I.kind = kind_of(g, x);
    int spt = (I.kind == 0) ? b->spt32 : b->spt16;
    if (x->LsE % spt != 0) spt = 1;
    I.spt = spt;
    I.TE = tile_of(x->LsE, x->nrhs, spt, b->split);
    const int L = x->LsE;
    I.lsp = (spt == 2 && L == x->LsP &&
             (L == 8 || L == 12 || L == 16 || L == 24 || L == 32 || L == 48 || L == 64)) ? L : 0;
    DhopParams& p = I.p;
    p = DhopParams{};
    p.U = g->d;
    p.in = x->d;
    p.in_norm = x->norm;
    p.out = o->d;
    p.out_norm = o->norm;
    p.nbr4 = g->lat->nbr4;
    p.nbr5 = nullptr;
    p.nsite = g->lat->nsite;
    p.LsE = x->LsE;
    p.LsP = x->LsP;
    p.Ls = g->lat->Ls;
    p.a5 = p.mf = 0.0;
    p.partials = nullptr;
    p.counter = nullptr;
    p.result = nullptr;
    p.err = nullptr;
    I.nthreads = unsigned(p.nsite * (p.LsE / spt));
    I.tile_threads = unsigned(p.nsite * (I.TE / spt));
    begin[k] = items;
    const unsigned nit = (I.nthreads + 31) / 32;
    item_inst.insert(item_inst.end(), nit, (unsigned short)k);
    items += nit;
  }
  b->total = items;
  if (item_inst.size() > b->item_cap) {
    if (b->d_item_inst) cudaFree(b->d_item_inst);
    b->d_item_inst = nullptr;
    b->item_cap = 0;
    GBDW_CUDA(dev_alloc((void**)&b->d_item_inst, item_inst.size() * sizeof(unsigned short)));
    b->item_cap = item_inst.size();
  }
  GBDW_CUDA(cudaMemcpyAsync(b->d_inst, hi.data(), sizeof(BatchInst) * n, cudaMemcpyHostToDevice, stream()));
  GBDW_CUDA(cudaMemcpyAsync(b->d_begin, begin.data(), sizeof(unsigned) * n, cudaMemcpyHostToDevice, stream()));
  GBDW_CUDA(cudaMemcpyAsync(b->d_item_inst, item_inst.data(), item_inst.size() * sizeof(unsigned short),
                            cudaMemcpyHostToDevice, stream()));
  int per_sm = 0;
  GBDW_CUDA(b->dag ? occupancy<1>(b->threads, &per_sm) : occupancy<0>(b->threads, &per_sm));
  if (per_sm < 1) per_sm = 1;
  b->grid = num_sms() * per_sm;
  if (unsigned(b->grid) > items) b->grid = int(items);
  // the host vectors above must outlive the queued copies
  GBDW_CUDA(cudaStreamSynchronize(stream()));
  cudaStream_t s = stream();
  GBDW_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  cudaMemsetAsync(b->d_next, 0, sizeof(unsigned), s);
  if (b->dag) launch<1>(b, s);
  else launch<0>(b, s);
  cudaError_t le = cudaGetLastError();
  cudaError_t ce = cudaStreamEndCapture(s, &b->graph);
  if (le != cudaSuccess) return cuda_fail(le, "k_batch capture");
  if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamEndCapture");
  GBDW_CUDA(cudaGraphInstantiate(&b->exec, b->graph, 0));
  return GBDW_OK;
}

int replay(gbdw_batch* b) {
  GBDW_CUDA(cudaGraphLaunch(b->exec, stream()));
  count_launch();  // the persistent kernel (the memset node is not a kernel of ours)
  return GBDW_OK;
}

// Times graph replays for each admissible shape and keeps the fastest.
int tune(gbdw_batch* b) {
  bool any16 = false, any32 = false;
  int max_split = 1;
  for (size_t i = 0; i < b->in.size(); ++i) {
    (b->in[i]->prec == GBDW_F16 ? any16 : any32) = true;
    max_split = std::max(max_split, b->in[i]->LsE / 2);
  }
  const int threads_c[] = {64, 128};
  const int spt_c[] = {2, 1};
  const int split_c[] = {1, 2, 4, 8};
  cudaEvent_t e0, e1;
  GBDW_CUDA(cudaEventCreate(&e0));
  GBDW_CUDA(cudaEventCreate(&e1));
  float best = 1e30f;
  int bt = b->threads, b32 = b->spt32, b16 = b->spt16, bsp = b->split;
  int st = GBDW_OK;
  for (int th : threads_c)
    for (int s32 : spt_c)
      for (int s16 : spt_c)
        for (int sp : split_c) {
          if (!any32 && s32 != spt_c[0]) continue;
          if (!any16 && s16 != spt_c[0]) continue;
          if (sp > max_split) continue;
          b->threads = th;
          b->spt32 = s32;
          b->spt16 = s16;
          b->split = sp;
          if ((st = build(b))) goto done;
          if ((st = replay(b))) goto done;
          cudaEventRecord(e0, stream());
          for (int r = 0; r < 3; ++r)
            if ((st = replay(b))) goto done;
          cudaEventRecord(e1, stream());
          cudaEventSynchronize(e1);
          float ms = 0.f;
          cudaEventElapsedTime(&ms, e0, e1);
          if (ms < best) {
            best = ms;
            bt = th;
            b32 = s32;
            b16 = s16;
            bsp = sp;
          }
        }
done:
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st) return st;
  b->threads = bt;
  b->spt32 = b32;
  b->spt16 = b16;
  b->split = bsp;
  return build(b);
}

}  // namespace

extern "C" {

int gbdw_batch_create(gbdw_batch** out, int n, const gbdw_gauge* const* gauges, gbdw_field* const* outs,
                      const gbdw_field* const* ins, int dag) {
  if (!out || n < 1 || n > 65535 || !gauges || !outs || !ins) {
    set_error("gbdw_batch_create: invalid arguments (1 to 65535 instances)");
    return GBDW_ERR_INVALID;
  }
  for (int i = 0; i < n; ++i) {
    const gbdw_gauge* g = gauges[i];
    const gbdw_field* x = ins[i];
    const gbdw_field* o = outs[i];
    if (!g || !x || !o || x == o || x->lat != g->lat || o->lat != g->lat || x->prec != o->prec || x->nrhs != o->nrhs ||
        kind_of(g, x) < 0 || !g->lat->fast) {
      set_error("gbdw_batch_create: instance " + std::to_string(i) +
                " needs FP32 (F32 gauge) or FP16 (F16/BF16 gauge) fields on a 4D-factorised lattice, out != in");
      return GBDW_ERR_INVALID;
    }
    if (double(g->lat->nsite) * x->LsE >= 4294967295.0) {
      set_error("gbdw_batch_create: instance too large");
      return GBDW_ERR_INVALID;
    }
  }
  if (int st = ensure_device()) return st;
  gbdw_batch* b = new gbdw_batch();
  b->g.assign(gauges, gauges + n);
  b->out.assign(outs, outs + n);
  b->in.assign(ins, ins + n);
  b->dag = dag ? 1 : 0;
  cudaError_t e = dev_alloc((void**)&b->d_inst, sizeof(BatchInst) * n);
  if (e == cudaSuccess) e = dev_alloc((void**)&b->d_begin, sizeof(unsigned) * n);
  if (e == cudaSuccess) e = dev_alloc((void**)&b->d_next, 64);
  if (e != cudaSuccess) {
    gbdw_batch_destroy(b);
    return cuda_fail(e, "cudaMalloc(batch)");
  }
  if (int st = tune(b)) {
    gbdw_batch_destroy(b);
    return st;
  }
  *out = b;
  return GBDW_OK;
}

int gbdw_batch_run(gbdw_batch* b) {
  if (!b || !b->exec) return GBDW_ERR_INVALID;
  return replay(b);
}

int gbdw_batch_destroy(gbdw_batch* b) {
  if (!b) return GBDW_OK;
  cudaStreamSynchronize(stream());
  release_graph(b);
  if (b->d_inst) cudaFree(b->d_inst);
  if (b->d_begin) cudaFree(b->d_begin);
  if (b->d_item_inst) cudaFree(b->d_item_inst);
  if (b->d_next) cudaFree(b->d_next);
  delete b;
  return GBDW_OK;
}

int gbdw_batch_info(const gbdw_batch* b, int64_t info[4]) {
  if (!b || !info) return GBDW_ERR_INVALID;
  info[0] = b->total;
  info[1] = b->grid;
  info[2] = b->threads;
  info[3] = b->exec ? 1 : 0;
  return GBDW_OK;
}

int gbdw_batch_set_shape(gbdw_batch* b, const int shape[4]) {
  if (!b || !shape || (shape[0] != 64 && shape[0] != 128) || shape[1] < 1 || shape[1] > 2 ||
      shape[2] < 1 || shape[2] > 2 || shape[3] < 1 || (shape[3] & (shape[3] - 1))) {
    set_error("gbdw_batch_set_shape: threads 64/128, slices per thread 1 or 2, split a power of two");
    return GBDW_ERR_INVALID;
  }
  b->threads = shape[0];
  b->spt32 = shape[1];
  b->spt16 = shape[2];
  b->split = shape[3];
  return build(b);
}

int gbdw_batch_shape(const gbdw_batch* b, int shape[4]) {
  if (!b || !shape) return GBDW_ERR_INVALID;
  shape[0] = b->threads;
  shape[1] = b->spt32;
  shape[2] = b->spt16;
  shape[3] = b->split;
  return GBDW_OK;
}

}  // extern "C"
