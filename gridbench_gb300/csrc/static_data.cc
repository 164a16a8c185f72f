// The reference's static-data exchange format (TableGenerate.cc:93-138): Grid dumps a doubled
// gauge field, a source spinor, the reference result Dhop(source) and the neighbour /
// permute tables of one lattice as C source, which bench.cc and bench_simple.cc compile in
// (bench.cc:55-88, bench_simple.cc:72-84).
//
//   static_data.h   const uint64_t nsite = <outer sites> ;   const int Ls = <Ls> ;  + extern decls
//   static_data.cc  double U_static[] = { <%16.8le entries>, 0};  (same for Phi_static,
//                   Psi_cpp_static), uint64_t nbr_static[] = { <0x%llx entries>, 0};,
//                   uint8_t prm_static[] = { <0x%x entries>, 0};
//
// Every array ends with a sentinel 0 that is not data.  Array lengths: U nsite*144*Nsimd,
// Phi and Psi nsite*Ls*24*Nsimd, nbr and prm nsite*Ls*8; Nsimd follows from the U length.
// The writer emits the same layout (so a file made here compiles into the reference's
// benchmarks), the reader accepts any whitespace between entries.
#include <cerrno>
#include <cinttypes>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gbdw.h"

namespace gbdw {
void set_error(const std::string& msg);  // context.cu: the message gbdw_last_error returns
}

namespace {

int fail(const std::string& m) {
  gbdw::set_error(m);
  return GBDW_ERR_INVALID;
}

bool slurp(const char* path, std::string* out) {
  FILE* f = fopen(path, "rb");
  if (!f) return false;
  char buf[1 << 16];
  size_t n;
  out->clear();
  while ((n = fread(buf, 1, sizeof buf, f)) > 0) out->append(buf, n);
  fclose(f);
  return true;
}

// Start of the entries of `name[] = {` in text, or npos.
size_t array_start(const std::string& text, const char* name) {
  const std::string key = std::string(name) + "[]";
  size_t p = text.find(key);
  if (p == std::string::npos) return p;
  p = text.find('{', p);
  return p == std::string::npos ? p : p + 1;
}

// Parses the comma-separated entries up to the closing brace; the last entry (the sentinel)
// is dropped.  Calls put(index, token_start) for the others and returns the data count, or
// -1 on a malformed array.
template <class Put>
int64_t parse_entries(const std::string& text, size_t pos, Put put) {
  const size_t close = text.find('}', pos);
  if (close == std::string::npos) return -1;
  int64_t n = 0;
  const char* s = text.c_str();
  size_t i = pos;
  std::vector<size_t> starts;
  while (i < close) {
    while (i < close && (s[i] == ' ' || s[i] == '\n' || s[i] == '\r' || s[i] == '\t')) ++i;
    if (i >= close) break;
    starts.push_back(i);
    const size_t comma = text.find(',', i);
    if (comma == std::string::npos || comma > close) break;  // the sentinel
    i = comma + 1;
  }
  if (starts.empty()) return -1;
  n = int64_t(starts.size()) - 1;
  for (int64_t k = 0; k < n; ++k)
    if (!put(k, s + starts[size_t(k)])) return -1;
  return n;
}

int64_t count_entries(const std::string& text, const char* name) {
  const size_t p = array_start(text, name);
  if (p == std::string::npos) return -1;
  return parse_entries(text, p, [](int64_t, const char*) { return true; });
}

bool header_values(const std::string& h, uint64_t* nsite, int* Ls) {
  const size_t a = h.find("nsite");
  const size_t b = h.find("Ls");
  if (a == std::string::npos || b == std::string::npos) return false;
  const size_t ea = h.find('=', a), eb = h.find('=', b);
  if (ea == std::string::npos || eb == std::string::npos) return false;
  char* end = nullptr;
  *nsite = strtoull(h.c_str() + ea + 1, &end, 10);
  if (end == h.c_str() + ea + 1) return false;
  *Ls = int(strtol(h.c_str() + eb + 1, &end, 10));
  return end != h.c_str() + eb + 1 && *nsite > 0 && *Ls > 0;
}

const char* kNames[5] = {"U_static", "Phi_static", "Psi_cpp_static", "nbr_static", "prm_static"};

}  // namespace

extern "C" {

int gbdw_static_data_info(const char* h_path, const char* cc_path, uint64_t* nsite, int* Ls, int* nsimd,
                          uint64_t counts[5]) {
  if (!h_path || !cc_path || !nsite || !Ls || !nsimd || !counts) return fail("gbdw_static_data_info: null argument");
  std::string h, cc;
  if (!slurp(h_path, &h)) return fail(std::string("cannot read ") + h_path);
  if (!slurp(cc_path, &cc)) return fail(std::string("cannot read ") + cc_path);
  if (!header_values(h, nsite, Ls)) return fail(std::string("no nsite / Ls constants in ") + h_path);
  for (int k = 0; k < 5; ++k) {
    const int64_t n = count_entries(cc, kNames[k]);
    if (n < 0) return fail(std::string("array ") + kNames[k] + " missing or malformed in " + cc_path);
    counts[k] = uint64_t(n);
  }
  const uint64_t ns = *nsite, L = uint64_t(*Ls);
  if (counts[0] % (ns * 144) != 0 || counts[0] == 0) return fail("U_static length is not nsite*144*Nsimd");
  *nsimd = int(counts[0] / (ns * 144));
  const uint64_t f = ns * L * 24 * uint64_t(*nsimd);
  if (counts[1] != f || counts[2] != f || counts[3] != ns * L * 8 || counts[4] != ns * L * 8)
    return fail("array lengths disagree with nsite, Ls and Nsimd");
  return GBDW_OK;
}

int gbdw_static_data_read(const char* cc_path, double* U, uint64_t nU, double* Phi, uint64_t nPhi, double* Psi,
                          uint64_t nPsi, uint64_t* nbr, uint64_t nnbr, uint8_t* prm, uint64_t nprm) {
  if (!cc_path) return fail("gbdw_static_data_read: null path");
  std::string cc;
  if (!slurp(cc_path, &cc)) return fail(std::string("cannot read ") + cc_path);
  double* dbl[3] = {U, Phi, Psi};
  const uint64_t cap[5] = {nU, nPhi, nPsi, nnbr, nprm};
  for (int k = 0; k < 5; ++k) {
    const size_t p = array_start(cc, kNames[k]);
    if (p == std::string::npos) return fail(std::string("array ") + kNames[k] + " missing");
    bool bad = false;
    int64_t n;
    if (k < 3) {
      double* dst = dbl[k];
      n = parse_entries(cc, p, [&](int64_t i, const char* t) {
        if (uint64_t(i) >= cap[k] || !dst) return false;
        char* end = nullptr;
        dst[i] = strtod(t, &end);
        return end != t;
      });
    } else if (k == 3) {
      n = parse_entries(cc, p, [&](int64_t i, const char* t) {
        if (uint64_t(i) >= cap[k] || !nbr) return false;
        char* end = nullptr;
        nbr[i] = strtoull(t, &end, 0);
        return end != t;
      });
    } else {
      n = parse_entries(cc, p, [&](int64_t i, const char* t) {
        if (uint64_t(i) >= cap[k] || !prm) return false;
        char* end = nullptr;
        const unsigned long v = strtoul(t, &end, 0);
        if (end == t || v > 255) return false;
        prm[i] = uint8_t(v);
        return true;
      });
    }
    bad = n < 0 || uint64_t(n) != cap[k];
    if (bad) return fail(std::string("array ") + kNames[k] + ": malformed, or its length differs from the buffer");
  }
  return GBDW_OK;
}

int gbdw_static_data_write(const char* h_path, const char* cc_path, uint64_t nsite, int Ls, int nsimd,
                           const double* U, const double* Phi, const double* Psi, const uint64_t* nbr,
                           const uint8_t* prm) {
  if (!h_path || !cc_path || nsite == 0 || Ls < 1 || nsimd < 1 || !U || !Phi || !Psi || !nbr || !prm)
    return fail("gbdw_static_data_write: invalid arguments");
  const uint64_t umax = nsite * 144 * uint64_t(nsimd), fmax = nsite * uint64_t(Ls) * 24 * uint64_t(nsimd),
                 nmax = nsite * uint64_t(Ls) * 8;
  FILE* f = fopen(cc_path, "w");
  if (!f) return fail(std::string("cannot write ") + cc_path);
  fprintf(f, "#include <stdint.h>\n");
  const double* arr[3] = {U, Phi, Psi};
  const uint64_t len[3] = {umax, fmax, fmax};
  for (int k = 0; k < 3; ++k) {
    fprintf(f, "double %s[] = { \n ", kNames[k]);
    for (uint64_t i = 0; i < len[k]; ++i) fprintf(f, "    %16.8le, \n", arr[k][i]);
    fprintf(f, "    0}; \n ");
  }
  fprintf(f, "uint64_t %s[] = { \n ", kNames[3]);
  for (uint64_t i = 0; i < nmax; ++i) fprintf(f, "    0x%" PRIx64 ", \n", nbr[i]);
  fprintf(f, "    0}; \n ");
  fprintf(f, "uint8_t %s[] = { \n ", kNames[4]);
  for (uint64_t i = 0; i < nmax; ++i) fprintf(f, "    0x%x, \n", unsigned(prm[i]));
  fprintf(f, "    0}; \n ");
  const bool ok = fclose(f) == 0;
  if (!ok) return fail(std::string("write failed: ") + cc_path);
  FILE* h = fopen(h_path, "w");
  if (!h) return fail(std::string("cannot write ") + h_path);
  fprintf(h, "#include <stdint.h>\n");
  fprintf(h, "const uint64_t nsite = %" PRIu64 " ; \n", nsite);
  fprintf(h, "const int Ls = %d ; \n", Ls);
  fprintf(h, "extern double   U_static[] ; \n");
  fprintf(h, "extern double   Phi_static[] ; \n");
  fprintf(h, "extern double   Psi_cpp_static[] ; \n");
  fprintf(h, "extern uint64_t nbr_static[] ; \n");
  fprintf(h, "extern uint8_t  prm_static[] ; \n");
  return fclose(h) == 0 ? GBDW_OK : fail(std::string("write failed: ") + h_path);
}

}  // extern "C"
