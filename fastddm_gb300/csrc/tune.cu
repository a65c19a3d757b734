// Launch configuration of the temporal kernels: a table of measured choices
// filled by the autotuner (timed candidates on first use of a problem class,
// or entries loaded from a committed table), and the occupancy model used
// when the table has no entry.
#include <map>
#include <mutex>
#include <tuple>
#include "fddm_b200.h"
#include "fddm_internal.h"

namespace fddm {
namespace {
std::mutex g_tune_mu;
std::map<std::tuple<int, int, int64_t, int64_t>, TemporalChoice> g_tune;  // (precision, mode, T, nlags)
bool g_autotune = false;
}  // namespace

bool tuned_temporal(int precision, int mode, int64_t T, int64_t nlags, TemporalChoice& out) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  auto it = g_tune.find(std::make_tuple(precision, mode, T, nlags));
  if (it == g_tune.end()) return false;
  out = it->second;
  return true;
}

void record_temporal(int precision, int mode, int64_t T, int64_t nlags, const TemporalChoice& c) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune[std::make_tuple(precision, mode, T, nlags)] = c;
}

bool autotune_enabled() {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  return g_autotune;
}

}  // namespace fddm

extern "C" {

int fddm_b200_set_autotune(int enable) {
  std::lock_guard<std::mutex> lk(fddm::g_tune_mu);
  fddm::g_autotune = enable != 0;
  return FDDM_OK;
}

int fddm_b200_tuning_set(int precision, int mode, uint64_t length, uint64_t nlags, int threads, int need_in_smem) {
  fddm::set_last_error("");
  if (precision < 0 || precision > 2 || (mode != FDDM_MODE_FFT && mode != FDDM_MODE_DIFF))
    return fddm::fail_with(FDDM_ERR_INVALID, "unknown precision or mode");
  if (threads != 128 && threads != 256 && threads != 512)
    return fddm::fail_with(FDDM_ERR_INVALID, "threads must be 128, 256 or 512");
  fddm::record_temporal(precision, mode, (int64_t)length, (int64_t)nlags, {threads, need_in_smem ? 1 : 0});
  return FDDM_OK;
}

int fddm_b200_tuning_get(int precision, int mode, uint64_t length, uint64_t nlags, int* threads, int* need_in_smem) {
  fddm::set_last_error("");
  if (!threads || !need_in_smem) return fddm::fail_with(FDDM_ERR_INVALID, "null pointer argument");
  fddm::TemporalChoice c{};
  if (!fddm::tuned_temporal(precision, mode, (int64_t)length, (int64_t)nlags, c))
    return fddm::fail_with(FDDM_ERR_INVALID, "no tuned entry for this problem class");
  *threads = c.threads;
  *need_in_smem = c.need_in_smem;
  return FDDM_OK;
}

uint64_t fddm_b200_tuning_count(void) {
  std::lock_guard<std::mutex> lk(fddm::g_tune_mu);
  return fddm::g_tune.size();
}

int fddm_b200_tuning_entry(uint64_t index, int* precision, int* mode, uint64_t* length, uint64_t* nlags, int* threads,
                           int* need_in_smem) {
  fddm::set_last_error("");
  if (!precision || !mode || !length || !nlags || !threads || !need_in_smem)
    return fddm::fail_with(FDDM_ERR_INVALID, "null pointer argument");
  std::lock_guard<std::mutex> lk(fddm::g_tune_mu);
  if (index >= fddm::g_tune.size()) return fddm::fail_with(FDDM_ERR_INVALID, "index out of range");
  auto it = fddm::g_tune.begin();
  std::advance(it, (long)index);
  *precision = std::get<0>(it->first);
  *mode = std::get<1>(it->first);
  *length = (uint64_t)std::get<2>(it->first);
  *nlags = (uint64_t)std::get<3>(it->first);
  *threads = it->second.threads;
  *need_in_smem = it->second.need_in_smem;
  return FDDM_OK;
}

}  // extern "C"
