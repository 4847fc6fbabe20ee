// Context, device workspace and error plumbing of libtnad.
#include <cstdlib>
#include <cstring>

#include "tnad_internal.h"

namespace tnad {

void fail(int code, const std::string& msg) { throw Error{code, msg}; }

Ten make_ten(double* p, std::initializer_list<int64_t> dims) {
  Ten t;
  t.p = p;
  t.nd = 0;
  for (int64_t d : dims) t.dim[t.nd++] = d;
  return t;
}

static const size_t kChunk = size_t(256) << 20;  // 256 MiB
static const size_t kAlign = 256;

void* Arena::alloc(size_t bytes) {
  bytes = (bytes + kAlign - 1) / kAlign * kAlign;
  if (bytes == 0) bytes = kAlign;
  while (cur_ < chunks_.size()) {
    Chunk& ch = chunks_[cur_];
    if (ch.used + bytes <= ch.cap) {
      void* p = ch.base + ch.used;
      ch.used += bytes;
      return p;
    }
    // does not fit: move on to the next chunk (stack order is kept by marks)
    if (cur_ + 1 < chunks_.size()) {
      ++cur_;
      chunks_[cur_].used = 0;
      continue;
    }
    break;
  }
  size_t cap = bytes > kChunk ? bytes : kChunk;
  char* p = nullptr;
  cudaError_t e = cudaMalloc(&p, cap);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    fail(TNAD_ERR_NOMEM, "workspace cudaMalloc of " + std::to_string(cap) + " bytes failed");
  }
  chunks_.push_back(Chunk{p, cap, bytes});
  cur_ = chunks_.size() - 1;
  return p;
}

Arena::Mark Arena::mark() const {
  if (chunks_.empty()) return Mark{0, 0};
  return Mark{cur_, chunks_[cur_].used};
}

void Arena::reset(const Mark& m) {
  if (chunks_.empty()) return;
  for (size_t i = m.chunk + 1; i < chunks_.size(); ++i) chunks_[i].used = 0;
  cur_ = m.chunk;
  chunks_[cur_].used = m.used;
}

void Arena::release_all() {
  for (auto& ch : chunks_) cudaFree(ch.base);
  chunks_.clear();
  cur_ = 0;
}

int64_t Arena::bytes_held() const {
  int64_t s = 0;
  for (auto& ch : chunks_) s += (int64_t)ch.cap;
  return s;
}

void check_launch(tnad_ctx* c, const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) fail(TNAD_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

}  // namespace tnad

using namespace tnad;

static void kt_clear(tnad_ctx* c);

extern "C" int tnad_version(void) { return 10000; }

extern "C" void tnad_opts_default(tnad_opts* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->prec = TNAD_PREC_FP64;
  o->solver = TNAD_SOLVER_FULL_SVD;
  o->adjoint = TNAD_ADJOINT_UNROLLED;
  o->fp_maxit = 200;
  o->fp_tol = 1e-10;
  o->ladder_tol = 1e-6;
  o->tape_budget = int64_t(16) << 30;
}

extern "C" int tnad_ctx_create(tnad_ctx** out, int device) {
  if (!out) return TNAD_ERR_ARG;
  *out = nullptr;
  tnad_ctx* c = new tnad_ctx();
  c->device = device;
  try {
    int ndev = 0;
    TNAD_CK(cudaGetDeviceCount(&ndev));
    TNAD_REQUIRE(device >= 0 && device < ndev, TNAD_ERR_ARG, "no such CUDA device");
    TNAD_CK(cudaSetDevice(device));
    cudaDeviceProp prop;
    TNAD_CK(cudaGetDeviceProperties(&prop, device));
    c->sm_count = prop.multiProcessorCount;
    c->tc_ok = (prop.major == 10);
    TNAD_CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    TNAD_CK(cudaMalloc(&c->d_red, 4096 * sizeof(double)));
    TNAD_CK(cudaMallocHost(&c->h_pin, 64 * sizeof(double)));
    TNAD_CK(cudaMalloc(&c->d_flag, 64 * sizeof(int)));
    TNAD_CK(cudaMallocHost(&c->h_flag, 64 * sizeof(int)));
    TNAD_CK(cudaMemsetAsync(c->d_flag, 0, 64 * sizeof(int), c->stream));
    if (const char* f = std::getenv("TNAD_EIG_POLISH")) c->eig_refine = std::strcmp(f, "jacobi") != 0;
    if (const char* f = std::getenv("TNAD_JACOBI_BLOCKS")) c->jacobi_blocks = std::strcmp(f, "0") != 0;
    if (const char* f = std::getenv("TNAD_TEST_FAULT")) {
      if (!std::strcmp(f, "tc_withhold")) c->fault_once = kFaultTcWithhold;
      if (!std::strcmp(f, "jacobi_cap")) c->fault_once = kFaultJacobiCap;
    }
  } catch (const Error& e) {
    int code = e.code;
    tnad_ctx_destroy(c);
    return code;
  }
  *out = c;
  return TNAD_OK;
}

extern "C" void tnad_ctx_destroy(tnad_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  c->ws.release_all();
  kt_clear(c);
  if (c->d_red) cudaFree(c->d_red);
  if (c->h_pin) cudaFreeHost(c->h_pin);
  if (c->d_flag) cudaFree(c->d_flag);
  if (c->h_flag) cudaFreeHost(c->h_flag);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

extern "C" const char* tnad_last_error(const tnad_ctx* c) { return c ? c->err.c_str() : "null context"; }

extern "C" int64_t tnad_ctx_workspace_bytes(const tnad_ctx* c) { return c ? c->ws.bytes_held() : 0; }

extern "C" int64_t tnad_ctx_kernel_launches(const tnad_ctx* c) { return c ? c->launches : 0; }

static void kt_clear(tnad_ctx* c) {
  for (auto& p : c->kt_ev) {
    cudaEventDestroy(p.first);
    cudaEventDestroy(p.second);
  }
  c->kt_ev.clear();
  c->kt_work = 0.0;
  c->kt_launches = 0;
}

extern "C" int tnad_ctx_kernel_timer(tnad_ctx* c, const char* name) {
  if (!c) return TNAD_ERR_ARG;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  kt_clear(c);
  c->ktimer = name ? name : "";
  return TNAD_OK;
}

extern "C" int tnad_ctx_kernel_timer_read(tnad_ctx* c, int64_t* launches, double* total_ms, double* work) {
  if (!c) return TNAD_ERR_ARG;
  cudaSetDevice(c->device);
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) return TNAD_ERR_CUDA;
  double ms = 0.0;
  for (auto& p : c->kt_ev) {
    float t = 0.f;
    if (cudaEventElapsedTime(&t, p.first, p.second) == cudaSuccess) ms += t;
  }
  if (launches) *launches = c->kt_launches;
  if (total_ms) *total_ms = ms;
  if (work) *work = c->kt_work;
  return TNAD_OK;
}

extern "C" void* tnad_ctx_stream(tnad_ctx* c) { return c ? (void*)c->stream : nullptr; }

// ---------------------------------------------------------------- phase trace
#include <cstdio>
#include <cstdlib>
#include <map>
#include <string>

namespace tnad {

PhaseTrace::PhaseTrace(tnad_ctx* c, const char* name) : c_(c), name_(name), on_(std::getenv("TNAD_TRACE") != nullptr) {}

void PhaseTrace::mark(const char* phase) {
  if (!on_) return;
  cudaEvent_t e;
  if (cudaEventCreate(&e) != cudaSuccess) return;
  cudaEventRecord(e, c_->stream);
  ev_.push_back({phase, e});
}

PhaseTrace::~PhaseTrace() {
  if (!on_ || ev_.empty()) return;
  mark("end");
  cudaEventSynchronize(ev_.back().second);
  std::map<std::string, std::pair<double, int>> acc;
  for (size_t i = 0; i + 1 < ev_.size(); ++i) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ev_[i].second, ev_[i + 1].second);
    auto& a = acc[ev_[i].first];
    a.first += ms;
    a.second += 1;
  }
  double tot = 0.0;
  for (auto& kv : acc) tot += kv.second.first;
  std::fprintf(stderr, "[tnad trace] %s: %.3f ms\n", name_, tot);
  for (auto& kv : acc)
    std::fprintf(stderr, "[tnad trace]   %-18s %9.3f ms  (%d)\n", kv.first.c_str(), kv.second.first, kv.second.second);
  for (auto& p : ev_) cudaEventDestroy(p.second);
}

}  // namespace tnad
