// Library-wide C-ABI pieces: version, thread-local error state and
// dimension validation.
#include <atomic>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "mb_internal.h"

namespace mb {

static thread_local char g_last_error[512] = "";

mb_status fail(mb_status s, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
  return s;
}

void clear_error() { g_last_error[0] = '\0'; }

mb_status check_dims(const mb_dims* d, bool need_beam) {
  if (d == nullptr) return fail(MB_ERR_NULL_PTR, "dims is NULL");
  const mb_dim* all[] = {&d->ntime, &d->na,    &d->nbl,   &d->nchan,   &d->npol,
                         &d->npolchan, &d->nsrc, &d->npsrc, &d->ngsrc, &d->nssrc,
                         &d->beam_lw, &d->beam_mh, &d->beam_nud};
  const char* names[] = {"ntime", "na",    "nbl",   "nchan",   "npol",    "npolchan", "nsrc",
                         "npsrc", "ngsrc", "nssrc", "beam_lw", "beam_mh", "beam_nud"};
  for (int i = 0; i < 13; ++i) {
    if (!dim_ok(*all[i]))
      return fail(MB_ERR_BAD_EXTENT,
                  "dimension %s: need lower <= upper, upper - lower <= local <= global "
                  "(got global %u local %u lower %u upper %u)",
                  names[i], all[i]->global_size, all[i]->local_size, all[i]->lower_extent,
                  all[i]->upper_extent);
  }
  if (d->npol.local_size != 4) return fail(MB_ERR_BAD_SHAPE, "npol must be 4 (got %u)", d->npol.local_size);
  if (d->npolchan.local_size != 4 * d->nchan.local_size)
    return fail(MB_ERR_BAD_SHAPE, "npolchan (%u) must equal 4 * nchan (%u)", d->npolchan.local_size,
                d->nchan.local_size);
  if (ext(d->npsrc) + ext(d->ngsrc) + ext(d->nssrc) != ext(d->nsrc))
    return fail(MB_ERR_BAD_SHAPE, "active nsrc extent (%u) must equal point + gaussian + sersic (%u)",
                ext(d->nsrc), ext(d->npsrc) + ext(d->ngsrc) + ext(d->nssrc));
  if (d->npsrc.local_size + d->ngsrc.local_size + d->nssrc.local_size != d->nsrc.local_size)
    return fail(MB_ERR_BAD_SHAPE, "local nsrc (%u) must equal point + gaussian + sersic (%u)",
                d->nsrc.local_size, d->npsrc.local_size + d->ngsrc.local_size + d->nssrc.local_size);
  if (need_beam && (d->beam_lw.local_size < 1 || d->beam_mh.local_size < 1 || d->beam_nud.local_size < 1))
    return fail(MB_ERR_BAD_SHAPE, "beam cube dimensions must be >= 1");
  return MB_OK;
}

// ---- launch accounting and per-kernel timing ---------------------------------
namespace {

struct TimedLaunch {
  const char* name;  // static string of the launch site
  cudaEvent_t start, stop;
};

std::atomic<uint64_t> g_launches{0};
std::atomic<bool> g_timing{false};
std::mutex g_timing_mutex;
std::vector<TimedLaunch> g_records;
std::vector<std::pair<cudaEvent_t, cudaEvent_t>> g_free_events;
std::vector<std::string> g_names;

}  // namespace

KernelScope::KernelScope(const char* name, cudaStream_t stream) : slot_(-1), stream_(stream) {
  g_launches.fetch_add(1, std::memory_order_relaxed);
  if (!g_timing.load(std::memory_order_relaxed)) return;
  std::lock_guard<std::mutex> lock(g_timing_mutex);
  std::pair<cudaEvent_t, cudaEvent_t> ev;
  if (!g_free_events.empty()) {
    ev = g_free_events.back();
    g_free_events.pop_back();
  } else if (cudaEventCreate(&ev.first) != cudaSuccess || cudaEventCreate(&ev.second) != cudaSuccess) {
    return;  // timing is best-effort; the launch itself proceeds
  }
  if (cudaEventRecord(ev.first, stream) != cudaSuccess) {
    g_free_events.push_back(ev);
    return;
  }
  slot_ = int(g_records.size());
  g_records.push_back({name, ev.first, ev.second});
}

KernelScope::~KernelScope() {
  if (slot_ < 0) return;
  std::lock_guard<std::mutex> lock(g_timing_mutex);
  if (slot_ < int(g_records.size())) cudaEventRecord(g_records[slot_].stop, stream_);
}

}  // namespace mb

extern "C" {

uint64_t mb_kernel_launches(void) { return mb::g_launches.load(); }

mb_status mb_kernel_timing(int enable) {
  mb::g_timing.store(enable != 0);
  return MB_OK;
}

mb_status mb_kernel_time(const char* name, double* total_ms, int64_t* launches) {
  MB_REQUIRE(total_ms, "total_ms");
  MB_REQUIRE(launches, "launches");
  std::lock_guard<std::mutex> lock(mb::g_timing_mutex);
  double ms = 0.0;
  int64_t n = 0;
  for (const auto& r : mb::g_records) {
    if (name != nullptr && std::strcmp(name, r.name) != 0) continue;
    MB_CUDA(cudaEventSynchronize(r.stop));
    float e = 0.f;
    MB_CUDA(cudaEventElapsedTime(&e, r.start, r.stop));
    ms += e;
    ++n;
  }
  *total_ms = ms;
  *launches = n;
  return MB_OK;
}

mb_status mb_kernel_timing_reset(void) {
  std::lock_guard<std::mutex> lock(mb::g_timing_mutex);
  for (const auto& r : mb::g_records) {
    MB_CUDA(cudaEventSynchronize(r.stop));
    mb::g_free_events.push_back({r.start, r.stop});
  }
  mb::g_records.clear();
  return MB_OK;
}

const char* mb_kernel_timing_name(int i) {
  std::lock_guard<std::mutex> lock(mb::g_timing_mutex);
  for (const auto& r : mb::g_records) {
    bool seen = false;
    for (const auto& x : mb::g_names) seen = seen || x == r.name;
    if (!seen) mb::g_names.push_back(r.name);
  }
  return (i >= 0 && i < int(mb::g_names.size())) ? mb::g_names[i].c_str() : nullptr;
}

const char* mb_version(void) { return "montblanc_gb300 0.1 (sm_103a)"; }

const char* mb_last_error_string(void) { return mb::g_last_error; }

const char* mb_status_string(mb_status s) {
  switch (s) {
    case MB_OK: return "MB_OK";
    case MB_ERR_NULL_PTR: return "MB_ERR_NULL_PTR";
    case MB_ERR_BAD_SHAPE: return "MB_ERR_BAD_SHAPE";
    case MB_ERR_BAD_EXTENT: return "MB_ERR_BAD_EXTENT";
    case MB_ERR_UNSUPPORTED_DTYPE: return "MB_ERR_UNSUPPORTED_DTYPE";
    case MB_ERR_CUDA: return "MB_ERR_CUDA";
    case MB_ERR_TIMEOUT: return "MB_ERR_TIMEOUT";
    case MB_ERR_WORKSPACE: return "MB_ERR_WORKSPACE";
    case MB_ERR_INVALID_ARG: return "MB_ERR_INVALID_ARG";
    case MB_ERR_UNSUPPORTED: return "MB_ERR_UNSUPPORTED";
  }
  return "MB_ERR_UNKNOWN";
}

}  // extern "C"
