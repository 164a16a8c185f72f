// Batched hopping term: many independent instances (each with its own lattice volume, Ls,
// right-hand sides, gauge field and storage precision FP32 or FP16) applied in ONE
// persistent launch that is captured once in a CUDA graph and replayed.
//
// The instances are cut into work items of one CTA's worth of threads (a thread owns
// `spt` consecutive innermost slices of one site).  A grid of (SMs x resident CTAs per SM)
// CTAs pulls items from a device counter with atomicAdd until the list is exhausted, so
// uneven volumes balance dynamically; the loop is bounded by the item count and never
// waits on another CTA.  The counter is reset by a memset node in the same graph.
// Launch shape (threads per CTA, slices per thread for each precision) is chosen by timing
// graph replays of the caller's own batch.
#include <algorithm>
#include <vector>

#include "common.cuh"
#include "dhop_kernel.cuh"

namespace gbdw {
namespace {

struct BatchInst {
  DhopParams p;
  unsigned item_begin;
  unsigned nthreads;  // nsite * LsE / spt
  int kind;           // 0: F32/F32, 1: F16/F16-gauge, 2: F16/BF16-gauge
  int spt;
};

template <int PIN, int GP, int DAG, int N>
__device__ __forceinline__ void batch_thread(const DhopParams& p, unsigned tid) {
  const unsigned G = unsigned(p.LsE) / N;
  const unsigned site = tid / G;
  const int s0 = int(tid - site * G) * N;
  using T = typename Arith<PIN>::T;
  cpx<T> acc[N][12];
  dhop_thread<PIN, GP, DAG, N>(p, site, s0, acc);
  store_spinor<PIN, N>(p.out, p.out_norm, site, s0, p.LsE, p.LsP, acc);
}

template <int DAG>
__global__ void __launch_bounds__(256) k_batch(const BatchInst* __restrict__ inst, int ninst, unsigned total,
                                               unsigned* next) {
  __shared__ unsigned item;
  __shared__ int which;
  for (;;) {
    if (threadIdx.x == 0) {
      item = atomicAdd(next, 1u);
      // instances are few: find the owner with a binary search over item_begin
      int lo = 0, hi = ninst - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (inst[mid].item_begin <= item) lo = mid;
        else hi = mid - 1;
      }
      which = lo;
    }
    __syncthreads();
    const unsigned it = item;
    const int k = which;
    __syncthreads();
    if (it >= total) break;
    const BatchInst& I = inst[k];
    const unsigned tid = (it - I.item_begin) * blockDim.x + threadIdx.x;
    if (tid < I.nthreads) {
      const DhopParams& p = I.p;
      if (I.kind == 0) {
        if (I.spt == 2) batch_thread<GBDW_F32, GBDW_F32, DAG, 2>(p, tid);
        else batch_thread<GBDW_F32, GBDW_F32, DAG, 1>(p, tid);
      } else if (I.kind == 1) {
        if (I.spt == 2) batch_thread<GBDW_F16, GBDW_F16, DAG, 2>(p, tid);
        else batch_thread<GBDW_F16, GBDW_F16, DAG, 1>(p, tid);
      } else {
        if (I.spt == 2) batch_thread<GBDW_F16, GBDW_BF16, DAG, 2>(p, tid);
        else batch_thread<GBDW_F16, GBDW_BF16, DAG, 1>(p, tid);
      }
    }
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
  BatchInst* d_inst = nullptr;
  unsigned* d_next = nullptr;
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

// Builds the work list for the current shape and captures [reset counter, persistent kernel].
int build(gbdw_batch* b) {
  release_graph(b);
  const int n = int(b->g.size());
  std::vector<BatchInst> hi(n);
  // largest instances first so the tail of the dynamic schedule is made of small items
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int c) {
    return b->in[a]->lat->nsite * b->in[a]->LsE > b->in[c]->lat->nsite * b->in[c]->LsE;
  });
  unsigned items = 0;
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
    DhopParams& p = I.p;
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
    I.item_begin = items;
    items += (I.nthreads + b->threads - 1) / b->threads;
  }
  b->total = items;
  GBDW_CUDA(cudaMemcpyAsync(b->d_inst, hi.data(), sizeof(BatchInst) * n, cudaMemcpyHostToDevice, stream()));
  int per_sm = 0;
  if (b->dag)
    GBDW_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch<1>, b->threads, 0));
  else
    GBDW_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch<0>, b->threads, 0));
  if (per_sm < 1) per_sm = 1;
  b->grid = num_sms() * per_sm;
  if (unsigned(b->grid) > items) b->grid = int(items);
  GBDW_CUDA(cudaStreamSynchronize(stream()));
  cudaStream_t s = stream();
  GBDW_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  cudaMemsetAsync(b->d_next, 0, sizeof(unsigned), s);
  if (b->dag) k_batch<1><<<b->grid, b->threads, 0, s>>>(b->d_inst, n, b->total, b->d_next);
  else k_batch<0><<<b->grid, b->threads, 0, s>>>(b->d_inst, n, b->total, b->d_next);
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
  for (size_t i = 0; i < b->in.size(); ++i) (b->in[i]->prec == GBDW_F16 ? any16 : any32) = true;
  const int threads_c[] = {64, 128, 256};
  const int spt_c[] = {1, 2};
  cudaEvent_t e0, e1;
  GBDW_CUDA(cudaEventCreate(&e0));
  GBDW_CUDA(cudaEventCreate(&e1));
  float best = 1e30f;
  int bt = b->threads, b32 = b->spt32, b16 = b->spt16;
  int st = GBDW_OK;
  for (int th : threads_c)
    for (int s32 : spt_c)
      for (int s16 : spt_c) {
        if (!any32 && s32 != spt_c[0]) continue;
        if (!any16 && s16 != spt_c[0]) continue;
        b->threads = th;
        b->spt32 = s32;
        b->spt16 = s16;
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
        }
      }
done:
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st) return st;
  b->threads = bt;
  b->spt32 = b32;
  b->spt16 = b16;
  return build(b);
}

}  // namespace

extern "C" {

int gbdw_batch_create(gbdw_batch** out, int n, const gbdw_gauge* const* gauges, gbdw_field* const* outs,
                      const gbdw_field* const* ins, int dag) {
  if (!out || n < 1 || !gauges || !outs || !ins) {
    set_error("gbdw_batch_create: invalid arguments");
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
  if (e == cudaSuccess) e = dev_alloc((void**)&b->d_next, 64);
  if (e != cudaSuccess) {
    if (b->d_inst) cudaFree(b->d_inst);
    delete b;
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

}  // extern "C"
