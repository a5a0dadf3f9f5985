// tuner.cu — see tuner.h.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <sys/stat.h>
#include <tuple>
#include <vector>

#include "engine.h"
#include "tuner.h"

namespace estl {

namespace {

struct Entry {
  PlanChoice choice;
  double ms = 0;
};

std::mutex g_mu;
std::map<std::tuple<std::string, long long, int>, Entry> g_cache;
bool g_loaded = false;

std::string gpu_name() {
  cudaDeviceProp prop;
  int dev = 0;
  cudaGetDevice(&dev);
  if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) return "unknown";
  std::string s = prop.name;
  for (char& ch : s)
    if (ch == '"' || ch == '\\') ch = '_';
  return s;
}

int batch_bucket(long long batch) {
  int b = 0;
  while ((2LL << b) <= batch) b++;
  return b;
}

long long json_int(const std::string& line, const char* key, long long dflt) {
  std::string k = std::string("\"") + key + "\":";
  size_t p = line.find(k);
  if (p == std::string::npos) return dflt;
  return std::strtoll(line.c_str() + p + k.size(), nullptr, 10);
}

std::string json_str(const std::string& line, const char* key) {
  std::string k = std::string("\"") + key + "\": \"";
  size_t p = line.find(k);
  if (p == std::string::npos) return "";
  size_t q = line.find('"', p + k.size());
  return line.substr(p + k.size(), q - p - k.size());
}

}  // namespace

std::string tuner_cache_path() {
  const char* env = std::getenv("ESTL_TUNE_CACHE");
  if (env && *env) return env;
  const char* home = std::getenv("HOME");
  return std::string(home && *home ? home : "/tmp") + "/.cache/estl_gb300/tune.jsonl";
}

std::string choice_to_json(const PlanChoice& c) {
  char buf[448];
  std::snprintf(buf, sizeof buf,
                "{\"mode\": %d, \"single_loge\": %d, \"single_logc\": %d, \"logn2\": %d, \"col_loge\": %d, "
                "\"col_logc\": %d, \"row_loge\": %d, \"row_logc\": %d, \"chunk\": %lld, \"pipe\": %d, "
                "\"logn3\": %d, \"single_logr\": %d, \"col_logr\": %d, \"row_logr\": %d, \"single_cluster\": %d}",
                c.mode, c.single_loge, c.single_logc, c.logn2, c.col_loge, c.col_logc, c.row_loge, c.row_logc, c.chunk,
                c.pipe, c.logn3, c.single_logr, c.col_logr, c.row_logr, c.single_cluster);
  return buf;
}

void tuner_load_cache() {
  std::lock_guard<std::mutex> g(g_mu);
  if (g_loaded) return;
  g_loaded = true;
  std::ifstream f(tuner_cache_path());
  std::string line;
  while (std::getline(f, line)) {
    std::string gpu = json_str(line, "gpu");
    long long n = json_int(line, "n", -1);
    int bb = (int)json_int(line, "batch_log2", -1);
    if (gpu.empty() || n < 1 || bb < 0) continue;
    Entry e;
    e.choice.mode = (int)json_int(line, "mode", 0);
    e.choice.single_loge = (int)json_int(line, "single_loge", -1);
    e.choice.single_logc = (int)json_int(line, "single_logc", -1);
    e.choice.logn2 = (int)json_int(line, "logn2", -1);
    e.choice.col_loge = (int)json_int(line, "col_loge", -1);
    e.choice.col_logc = (int)json_int(line, "col_logc", -1);
    e.choice.row_loge = (int)json_int(line, "row_loge", -1);
    e.choice.row_logc = (int)json_int(line, "row_logc", -1);
    e.choice.chunk = json_int(line, "chunk", 0);
    e.choice.pipe = (int)json_int(line, "pipe", 0);
    e.choice.logn3 = (int)json_int(line, "logn3", -1);
    e.choice.single_logr = (int)json_int(line, "single_logr", -1);
    e.choice.col_logr = (int)json_int(line, "col_logr", -1);
    e.choice.row_logr = (int)json_int(line, "row_logr", -1);
    e.choice.single_cluster = (int)json_int(line, "single_cluster", -1);
    g_cache[{gpu, n, bb}] = e;  // later lines win
  }
}

bool tuner_lookup(long long n, long long batch, PlanChoice* out) {
  std::lock_guard<std::mutex> g(g_mu);
  auto it = g_cache.find({gpu_name(), n, batch_bucket(batch)});
  if (it == g_cache.end()) return false;
  *out = it->second.choice;
  return true;
}

void tuner_store(long long n, long long batch, const PlanChoice& c, double ms) {
  std::lock_guard<std::mutex> g(g_mu);
  std::string gpu = gpu_name();
  int bb = batch_bucket(batch);
  g_cache[{gpu, n, bb}] = Entry{c, ms};
  std::string path = tuner_cache_path();
  // mkdir -p of the cache directory
  for (size_t p = 1; p < path.size(); ++p)
    if (path[p] == '/') mkdir(path.substr(0, p).c_str(), 0755);
  std::ofstream f(path, std::ios::app);
  if (!f) return;
  std::string cj = choice_to_json(c);
  f << "{\"gpu\": \"" << gpu << "\", \"n\": " << n << ", \"batch_log2\": " << bb << ", \"ms\": " << ms << ", "
    << cj.substr(1) << "\n";
}

}  // namespace estl

using namespace estl;

extern "C" estl_status estl_autotune(int64_t n, int64_t batch, int iters, char* result_json, size_t len) {
  estl_status s = require_init();
  if (s != ESTL_OK) return s;
  if (iters < 1) iters = 5;
  std::vector<PlanChoice> cands = plan_candidates(n, batch);
  if (cands.empty()) return fail(ESTL_UNSUPPORTED_SIZE, "no candidate plans for n = %lld", (long long)n);
  std::vector<Plan1D> plans;
  long long max_scratch = 0;
  for (const PlanChoice& c : cands) {
    Plan1D p;
    std::string err;
    if (!make_plan(n, batch, c, &p, &err)) continue;
    max_scratch = std::max(max_scratch, p.scratch_elems);
    plans.push_back(p);
  }
  const size_t bytes = (size_t)(n * batch) * sizeof(cf32);
  cf32 *in = nullptr, *out = nullptr, *scr = nullptr;
  if ((s = dev_alloc((void**)&in, bytes, "autotune input")) != ESTL_OK) return s;
  if ((s = dev_alloc((void**)&out, bytes, "autotune output")) != ESTL_OK) {
    dev_free(in, bytes);
    return s;
  }
  if ((s = dev_alloc((void**)&scr, (size_t)max_scratch * sizeof(cf32), "autotune scratch")) != ESTL_OK) {
    dev_free(in, bytes);
    dev_free(out, bytes);
    return s;
  }
  cudaMemset(in, 0, bytes);
  cudaStream_t st;
  cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  double best_ms = 1e30;
  const Plan1D* best = nullptr;
  std::vector<std::pair<double, const Plan1D*>> timed;
  for (const Plan1D& p : plans) {
    s = launch_steps(p, in, out, scr, 1.f, st);
    if (s != ESTL_OK) continue;
    launch_steps(p, in, out, scr, 1.f, st);
    cudaEventRecord(e0, st);
    for (int i = 0; i < iters; ++i) launch_steps(p, in, out, scr, 1.f, st);
    cudaEventRecord(e1, st);
    if (cudaEventSynchronize(e1) != cudaSuccess) {
      s = check_cuda(cudaGetLastError(), "autotune run");
      break;
    }
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    ms /= iters;
    if (take_bulk_wait_error() != ESTL_OK) continue;  // a bounded wait gave up: not a usable configuration
    timed.push_back({ms, &p});
    if (ms < best_ms) {
      best_ms = ms;
      best = &p;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(st);
  dev_free(in, bytes);
  dev_free(out, bytes);
  dev_free(scr, (size_t)max_scratch * sizeof(cf32));
  if (!best) return s != ESTL_OK ? s : fail(ESTL_DEVICE_ERROR, "no candidate plan ran");
  tuner_store(n, batch, best->choice, best_ms);
  if (result_json && len) {
    std::string j = std::string("{\"n\": ") + std::to_string((long long)n) + ", \"batch\": " +
                    std::to_string((long long)batch) + ", \"candidates\": " + std::to_string(plans.size()) +
                    ", \"best_ms\": " + std::to_string(best_ms) + ", \"choice\": " + choice_to_json(best->choice) +
                    ", \"plan\": " + best->describe() + ", \"fastest\": [";
    std::sort(timed.begin(), timed.end(),
              [](const std::pair<double, const Plan1D*>& a, const std::pair<double, const Plan1D*>& b) {
                return a.first < b.first;
              });
    for (size_t i = 0; i < timed.size() && i < 8; ++i)
      j += std::string(i ? ", " : "") + "{\"ms\": " + std::to_string(timed[i].first) +
           ", \"choice\": " + choice_to_json(timed[i].second->choice) + "}";
    j += "]}";
    std::snprintf(result_json, len, "%s", j.c_str());
  }
  return ESTL_OK;
}
