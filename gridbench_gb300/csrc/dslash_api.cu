// Drop-in replacement for GridBench's kernel seam
//   template<class Simd> double dslash_kernel(int nrep, Simd* Up, Simd* outp, Simd* inp,
//                                             uint64_t* nbr, uint64_t nsite, uint64_t Ls, uint8_t* prm)
// (WilsonKernelsHand.h:17-18,25-26; called from bench.cc:148-164).
//
// Same arguments and meaning: reference-layout gauge field, input and output spinors with
// Nsimd lanes, the TableGenerate neighbour/permute tables, nsite outer sites, nrep
// repetitions.  Buffers may live on the host or the device.  The table is validated and
// reduced to a 4D table, the fields are converted once into the GB300 layout, the hopping
// term runs nrep times, and the result is converted back once.  The returned time covers
// repetitions 1..nrep-1 as in WilsonKernelsHandCpu.h:407-450 (device time from CUDA events
// instead of a host clock).  Errors come back as a status; nothing exits the process
// (unlike Macros.h:47-51).
#include "common.cuh"

namespace gbdw {
int lattice_from_table_impl(gbdw_lattice** out, uint64_t nouter, int Ls, int nsimd, const uint64_t* nbr,
                            const uint8_t* prm, bool force_general);
}

using namespace gbdw;

namespace {
struct Owned {
  gbdw_lattice* lat = nullptr;
  gbdw_gauge* g = nullptr;
  gbdw_field* in = nullptr;
  gbdw_field* out = nullptr;
  cudaEvent_t a = nullptr, b = nullptr;
  ~Owned() {
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    gbdw_field_destroy(out);
    gbdw_field_destroy(in);
    gbdw_gauge_destroy(g);
    gbdw_lattice_destroy(lat);
  }
};
}  // namespace

extern "C" int gbdw_dslash_kernel(int nrep, int prec, int nsimd, const void* U, void* out, const void* in,
                                  const uint64_t* nbr, uint64_t nsite, uint64_t Ls, const uint8_t* prm, int dag,
                                  double* usec) {
  if (nrep < 1 || !U || !out || !in || !nbr || nsite == 0 || Ls == 0 || Ls > 4096 ||
      (prec != GBDW_F64 && prec != GBDW_F32)) {
    set_error("gbdw_dslash_kernel: invalid arguments (nrep >= 1, non-null buffers, prec F64 or F32)");
    return GBDW_ERR_INVALID;
  }
  if (int st = ensure_device()) return st;
  Owned o;
  if (int st = lattice_from_table_impl(&o.lat, nsite, int(Ls), nsimd, nbr, prm, false)) return st;
  if (int st = gbdw_gauge_create(&o.g, o.lat, prec, U, prec)) return st;
  if (int st = gbdw_field_create(&o.in, o.lat, prec, 1)) return st;
  if (int st = gbdw_field_create(&o.out, o.lat, prec, 1)) return st;
  if (int st = gbdw_field_import(o.in, 0, in, prec)) return st;
  GBDW_CUDA(cudaEventCreate(&o.a));
  GBDW_CUDA(cudaEventCreate(&o.b));
  if (nrep == 1) GBDW_CUDA(cudaEventRecord(o.a, stream()));
  for (int rep = 0; rep < nrep; ++rep) {
    if (rep == 1) GBDW_CUDA(cudaEventRecord(o.a, stream()));
    if (int st = gbdw_dhop(o.g, o.out, o.in, dag)) return st;
  }
  GBDW_CUDA(cudaEventRecord(o.b, stream()));
  if (int st = gbdw_field_export(o.out, 0, out, prec)) return st;
  GBDW_CUDA(cudaEventSynchronize(o.b));
  float ms = 0.f;
  GBDW_CUDA(cudaEventElapsedTime(&ms, o.a, o.b));
  if (usec) *usec = double(ms) * 1000.0;
  GBDW_CUDA(cudaStreamSynchronize(stream()));
  return GBDW_OK;
}
