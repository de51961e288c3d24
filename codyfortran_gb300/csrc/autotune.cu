// autotune.cu -- tile autotuner of the engine (no counterpart in the reference).
//
// The set-up heuristics pick the fixed-point GEMM tiles (N-tile width,
// compact two-CTAs-per-SM or wide configuration, K splits: fx_tile_n /
// fx_split_count) and the blocks per trajectory of the Lanczos reductions
// from the sizes alone.  The tuner times the candidates on the context's own
// shapes and operands with CUDA events on the context stream and keeps the
// fastest:
//   * each of the three contractions W = V S, Z = W R'' and h2 = S^T W on its
//     own (GEMM plus its K-split reduction), every instantiated tile
//     configuration of its slice count at every K split the partial buffers
//     hold and the digits' exact range allows;
//   * the Lanczos family of one fixed-order SIL half step at half, one and two
//     times the heuristic's blocks per trajectory (as far as the partials hold).
// The fixed-point contractions are exact sums of digit products, so the tile
// choice does not change their results; a K split adds one FP64 rounding per
// partial, and the Lanczos block count changes the order of the FP64 partial
// sums of the reductions.
//
// Winners are kept in a JSON-lines cache, one object per shape key:
//   {"key": "...", "W": [bn, compact, splits], "Z": [...], "H2": [...], "lz_blocks": n}
// The key holds the precision, the device name and SM count, the Krylov
// order and window, the number of trajectories and a 64-bit FNV-1a hash of
// every trajectory's sizes, so a cache entry is reused only for the same
// batch shapes on the same kind of GPU.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>

#include "common.cuh"

namespace {

const char* kGemmName[3] = {"W", "Z", "H2"};

std::string tune_key(const cgpu_ctx* c) {
  uint64_t h = 1469598103934665603ull;
  auto mix = [&](long long v) {
    for (int i = 0; i < 8; i++) {
      h ^= (uint64_t)((v >> (8 * i)) & 0xFF);
      h *= 1099511628211ull;
    }
  };
  for (const TrajShape& t : c->shape_h) {
    mix(t.nG); mix(t.nOS); mix(t.nC); mix(t.nPairs); mix(t.Kg); mix(t.Kp); mix(t.vRow); mix(t.vRoot);
  }
  mix(c->fxShared);
  int dev = 0;
  cudaDeviceProp prop;
  std::memset(&prop, 0, sizeof(prop));
  if (cudaGetDevice(&dev) == cudaSuccess) cudaGetDeviceProperties(&prop, dev);
  char buf[512];
  std::snprintf(buf, sizeof(buf), "prec=%d;dev=%s;sms=%d;krylov=%d;window=%d;nb=%d;shape=%016llx", c->precision,
                prop.name, c->numSms, c->maxKrylov, c->krylovWindow, c->nb, (unsigned long long)h);
  return buf;
}

// Reads the entry of `key` from the cache file into t[10]; false if absent.
bool cache_read(const std::string& path, const std::string& key, int* t) {
  std::ifstream f(path);
  if (!f) return false;
  const std::string tag = "\"key\": \"" + key + "\"";
  std::string line;
  while (std::getline(f, line)) {
    if (line.find(tag) == std::string::npos) continue;
    int v[10];
    bool ok = true;
    for (int g = 0; g < 3 && ok; g++) {
      const std::string k = std::string("\"") + kGemmName[g] + "\": [";
      size_t p = line.find(k);
      ok = p != std::string::npos &&
           std::sscanf(line.c_str() + p + k.size(), "%d, %d, %d", &v[3 * g], &v[3 * g + 1], &v[3 * g + 2]) == 3;
    }
    size_t p = line.find("\"lz_blocks\": ");
    ok = ok && p != std::string::npos && std::sscanf(line.c_str() + p + 13, "%d", &v[9]) == 1;
    if (ok) {
      std::memcpy(t, v, sizeof(v));
      return true;
    }
  }
  return false;
}

// Replaces (or adds) the entry of `key`; written to a temporary file and renamed.
void cache_write(const std::string& path, const std::string& key, const int* t) {
  std::vector<std::string> keep;
  {
    std::ifstream f(path);
    std::string line;
    const std::string tag = "\"key\": \"" + key + "\"";
    while (f && std::getline(f, line))
      if (!line.empty() && line.find(tag) == std::string::npos) keep.push_back(line);
  }
  char buf[1024];
  std::snprintf(buf, sizeof(buf), "{\"key\": \"%s\", \"W\": [%d, %d, %d], \"Z\": [%d, %d, %d], \"H2\": [%d, %d, %d], "
                "\"lz_blocks\": %d}", key.c_str(), t[0], t[1], t[2], t[3], t[4], t[5], t[6], t[7], t[8], t[9]);
  keep.push_back(buf);
  const std::string tmp = path + ".tmp";
  {
    std::ofstream o(tmp, std::ios::trunc);
    if (!o) throw std::string("autotune: cannot write the cache file ") + tmp;
    for (const std::string& l : keep) o << l << "\n";
  }
  if (std::rename(tmp.c_str(), path.c_str()) != 0) throw std::string("autotune: cannot rename the cache file to ") + path;
}

void lz_candidates(const cgpu_ctx* c, std::vector<int>& out) {
  out.clear();
  for (int v : {c->lzBlocksHeur / 2, c->lzBlocksHeur, 2 * c->lzBlocksHeur}) {
    v = std::max(1, std::min(v, c->lzBlocksCap));
    if (std::find(out.begin(), out.end(), v) == out.end()) out.push_back(v);
  }
}

}  // namespace

void tiles_get(const cgpu_ctx* c, int* t) {
  if (!fx_tiles_get(c, t))
    for (int i = 0; i < 9; i++) t[i] = 0;
  t[9] = c->lzBlocks;
}

void tiles_set(cgpu_ctx* c, const int* t) {
  if (t[9] < 1 || t[9] > c->lzBlocksCap) throw std::string("tiles: Lanczos blocks per trajectory out of range");
  int cur[10];
  tiles_get(c, cur);
  bool gemm = false;
  for (int i = 0; i < 9; i++) gemm |= cur[i] != t[i];
  if (gemm) {
    if (!fx_tiles_get(c, cur)) throw std::string("tiles: GEMM tiles exist only in the fixed-point forms");
    fx_tiles_set(c, t);
  }
  c->lzBlocks = t[9];
  drop_step_graph(c);
}

// Tunes (or loads from the cache) and applies the tile table; report receives a
// JSON object with the source, the key, the candidates timed and the choice.
void autotune_run(cgpu_ctx* c, const char* cachePath, int force, std::string& report) {
  const std::string key = tune_key(c);
  int t[10];
  std::ostringstream js;
  js.precision(5);
  if (!force && cachePath && cache_read(cachePath, key, t)) {
    tiles_set(c, t);
    js << "{\"source\": \"cache\", \"key\": \"" << key << "\"";
  } else {
    tiles_get(c, t);
    js << "{\"source\": \"tuned\", \"key\": \"" << key << "\"";
    // the operands of the contractions: one NonLin derivative of the resident states
    if (c->method != CGPU_METHOD_TDCI) {
      td_device_public(c, CGPU_TD_NONLIN, c->dstate_d, c->state_d, 0.0);
      CODY_CUDA(cudaStreamSynchronize(c->stream));
    }
    int cur[9];
    if (fx_tiles_get(c, cur)) {
      for (int g = 0; g < 3; g++) {
        std::vector<std::array<int, 3>> cands;
        fx_tile_candidates(c, g, cands);
        double best = 1e300;
        int bestIdx = -1;
        js << ", \"" << kGemmName[g] << "_candidates\": [";
        for (size_t i = 0; i < cands.size(); i++) {
          int trial[9];
          std::memcpy(trial, t, sizeof(trial));
          trial[3 * g] = cands[i][0];
          trial[3 * g + 1] = cands[i][1];
          trial[3 * g + 2] = cands[i][2];
          fx_tiles_set(c, trial);
          const double ms = fx_time_contraction(c, g, 3);
          js << (i ? ", " : "") << "[" << cands[i][0] << ", " << cands[i][1] << ", " << cands[i][2] << ", " << ms
             << "]";
          if (ms < best) {
            best = ms;
            bestIdx = (int)i;
          }
        }
        js << "]";
        if (bestIdx >= 0) {
          t[3 * g] = cands[bestIdx][0];
          t[3 * g + 1] = cands[bestIdx][1];
          t[3 * g + 2] = cands[bestIdx][2];
        }
        fx_tiles_set(c, t);
      }
    }
    if (c->method != CGPU_METHOD_TDCI) {
      std::vector<int> lz;
      lz_candidates(c, lz);
      double best = 1e300;
      js << ", \"lz_candidates\": [";
      for (size_t i = 0; i < lz.size(); i++) {
        c->lzBlocks = lz[i];
        time_sil_lanczos(c, c->maxKrylov);  // warm-up
        const double ms = time_sil_lanczos(c, c->maxKrylov);
        js << (i ? ", " : "") << "[" << lz[i] << ", " << ms << "]";
        if (ms < best) {
          best = ms;
          t[9] = lz[i];
        }
      }
      js << "]";
    }
    tiles_set(c, t);
    if (cachePath && *cachePath) cache_write(cachePath, key, t);
  }
  js << ", \"tiles\": {\"W\": [" << t[0] << ", " << t[1] << ", " << t[2] << "], \"Z\": [" << t[3] << ", " << t[4]
     << ", " << t[5] << "], \"H2\": [" << t[6] << ", " << t[7] << ", " << t[8] << "], \"lz_blocks\": " << t[9] << "}}";
  report = js.str();
}
