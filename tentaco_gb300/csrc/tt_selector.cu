// tt_selector.cu -- the learned variant selector: model file, inference on the
// device (the network of tt_mlp.cu) and the ranked variant list a plan tries.
#include <cuda_runtime.h>
#include <dlfcn.h>
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>
#include "tt_internal.h"
#include "tt_plan.h"
#include "../../include/tentaco/tentaco_gen.h"
#include "../../include/tentaco/tentaco_select.h"

namespace tt {
namespace {

struct Model {
  int storage = 0;  // 0: FP32 storage plans, 1: 16-bit storage plans
  float mean[TT_MLP_IN], sd[TT_MLP_IN];
  float lo[TT_MLP_IN], hi[TT_MLP_IN];  // feature range of the training tensors
  std::vector<float> params;
};

// One model set per tensor order (three and four modes), each with its own
// default file beside the library.
struct ModelSet {
  std::vector<Model> models;
  int nout = 0;
  bool tried_default = false;
};
std::mutex g_mu;
ModelSet g_sets[2];  // [0]: three modes, [1]: four modes
int set_index(int order) { return order == 4 ? 1 : order == 3 ? 0 : -1; }

std::string default_model_path(int order = 3) {
  const char* name = order == 4 ? "/selector_model_o4.bin" : "/selector_model.bin";
  Dl_info info;
  if (dladdr((void*)&tt_selector_models, &info) && info.dli_fname) {
    std::string p(info.dli_fname);
    const size_t k = p.rfind('/');
    return (k == std::string::npos ? std::string(".") : p.substr(0, k)) + name;
  }
  return name + 1;
}

// File layout (little-endian): "TTSEL001", int32 {version, inputs, hidden, outputs,
// models}, (version 3) int32 tensor order, then per model: int32 storage, float
// mean[inputs], sd[inputs], (versions 2 and 3) lo[inputs], hi[inputs], params.
// Version 1 files carry no training range and count every tensor as inside it;
// versions 1 and 2 hold three-mode models.
tt_status load_file(const std::string& path, std::vector<Model>& out, int& nout, int& order) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return set_error(TT_ERR_INVALID_ARGUMENT, "selector model %s: cannot open", path.c_str());
  auto rd = [&](void* p, size_t n) { return std::fread(p, 1, n, f) == n; };
  char magic[8];
  int32_t hdr[5];
  bool ok = rd(magic, 8) && std::memcmp(magic, "TTSEL001", 8) == 0 && rd(hdr, sizeof(hdr));
  ok = ok && hdr[0] >= 1 && hdr[0] <= 3 && hdr[1] == TT_MLP_IN && hdr[2] == TT_MLP_HIDDEN && hdr[3] > 0 &&
       hdr[3] <= 4096 && hdr[4] > 0 && hdr[4] <= 8;
  int32_t ord = 3;
  if (ok && hdr[0] == 3) ok = rd(&ord, 4) && set_index(ord) >= 0;
  std::vector<Model> ms;
  if (ok) {
    const int64_t np = tt_mlp_num_params(hdr[3]);
    for (int i = 0; i < hdr[4] && ok; i++) {
      Model m;
      int32_t storage = 0;
      m.params.resize((size_t)np);
      ok = rd(&storage, 4) && rd(m.mean, sizeof(m.mean)) && rd(m.sd, sizeof(m.sd));
      if (hdr[0] >= 2) {
        ok = ok && rd(m.lo, sizeof(m.lo)) && rd(m.hi, sizeof(m.hi));
      } else {
        std::fill(m.lo, m.lo + TT_MLP_IN, -std::numeric_limits<float>::infinity());
        std::fill(m.hi, m.hi + TT_MLP_IN, std::numeric_limits<float>::infinity());
      }
      ok = ok && rd(m.params.data(), sizeof(float) * (size_t)np);
      m.storage = storage;
      for (int k = 0; k < TT_MLP_IN && ok; k++) ok = std::isfinite(m.mean[k]) && m.sd[k] > 0.f;
      ms.push_back(std::move(m));
    }
    char extra;
    ok = ok && std::fread(&extra, 1, 1, f) == 0;  // nothing after the last model
  }
  std::fclose(f);
  if (!ok) return set_error(TT_ERR_INVALID_ARGUMENT, "selector model %s: malformed", path.c_str());
  out = std::move(ms);
  nout = hdr[3];
  order = ord;
  return TT_OK;
}

// The model for a storage class and tensor order, loading that order's default
// file on first use.
const Model* model_for(int storage, int order, int& nout) {
  const int si = set_index(order);
  if (si < 0) return nullptr;
  std::lock_guard<std::mutex> lk(g_mu);
  ModelSet& set = g_sets[si];
  if (set.models.empty() && !set.tried_default) {
    set.tried_default = true;
    std::vector<Model> ms;
    int n = 0, ord = 0;
    if (load_file(default_model_path(order), ms, n, ord) == TT_OK && ord == order) {
      set.models = std::move(ms);
      set.nout = n;
    }
    clear_error();
  }
  for (const Model& m : set.models)
    if (m.storage == storage) { nout = set.nout; return &m; }
  return nullptr;
}

int storage_class(int prec) { return prec == (int)TT_PREC_FP32 ? 0 : 1; }

// Scores of every variant for tensor B (device inference).  Invalid variants: +inf.
// in_range (optional): whether every feature lies inside the training range.
tt_status scores_for(const taco_tensor_t* B, int order, int rank, int prec, std::vector<float>& scores,
                     bool* in_range = nullptr) {
  if (order != 3 && order != 4) return set_error(TT_ERR_UNSUPPORTED, "the selector covers 3- and 4-mode tensors");
  int nout = 0;
  const Model* m = model_for(storage_class(prec), order, nout);
  if (!m) return set_error(TT_ERR_UNSUPPORTED, "no selector model for this storage precision");
  float f[TT_MLP_IN];
  tt_status s = tt_csf_features(B, rank, f);
  if (s != TT_OK) return s;
  if (in_range) {
    *in_range = true;
    for (int k = 0; k < TT_MLP_IN; k++) *in_range = *in_range && f[k] >= m->lo[k] && f[k] <= m->hi[k];
  }
  for (int k = 0; k < TT_MLP_IN; k++) f[k] = (f[k] - m->mean[k]) / m->sd[k];
  const int64_t np = (int64_t)m->params.size();
  const int64_t ns = tt_mlp_scratch_floats(1, nout);
  float* d = nullptr;
  const size_t total = (size_t)(np + TT_MLP_IN + ns + nout);
  if (device_pool_alloc((void**)&d, total * sizeof(float), nullptr) != cudaSuccess)
    return set_error(TT_ERR_OUT_OF_MEMORY, "selector inference buffers");
  float* dp = d;
  float* dx = dp + np;
  float* dsc = dx + TT_MLP_IN;
  float* dout = dsc + ns;
  std::vector<float> out((size_t)nout);
  cudaError_t e = cudaMemcpy(dp, m->params.data(), sizeof(float) * (size_t)np, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dx, f, sizeof(f), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    s = tt_mlp_forward(dp, nout, dx, 1, dsc, dout, nullptr);
    if (s == TT_OK) e = cudaMemcpy(out.data(), dout, sizeof(float) * (size_t)nout, cudaMemcpyDeviceToHost);
  }
  device_pool_free(d, nullptr);
  cudaStreamSynchronize(nullptr);
  if (s != TT_OK) return s;
  if (e != cudaSuccess) return set_error(TT_ERR_CUDA, "selector inference: %s", cudaGetErrorString(e));
  const int nv = tt_num_variants();
  scores.assign((size_t)nv, std::numeric_limits<float>::infinity());
  for (int v = 0; v < nv && v < nout; v++)
    if (variant_valid(v, order, rank, prec)) scores[(size_t)v] = out[(size_t)v];
  return TT_OK;
}

}  // namespace

// Variants ordered by predicted time (valid ones only); empty when no model applies.
// in_range: whether the tensor's features lie inside the model's training range.
tt_status selector_rank(const tt_plan* p, const taco_tensor_t* B, std::vector<int>& ranked, bool* in_range) {
  ranked.clear();
  std::vector<float> sc;
  tt_status s = scores_for(B, p->order, p->rank, p->prec, sc, in_range);
  if (s != TT_OK) return s;
  for (int v = 0; v < (int)sc.size(); v++)
    if (std::isfinite(sc[(size_t)v])) ranked.push_back(v);
  std::stable_sort(ranked.begin(), ranked.end(), [&](int x, int y) { return sc[(size_t)x] < sc[(size_t)y]; });
  return TT_OK;
}

}  // namespace tt

using namespace tt;

TT_EXPORT tt_status tt_selector_load(const char* path) {
  clear_error();
  std::vector<Model> ms;
  int n = 0, ord = 3;
  tt_status s = load_file(path ? std::string(path) : default_model_path(), ms, n, ord);
  if (s != TT_OK) return s;
  std::lock_guard<std::mutex> lk(g_mu);
  ModelSet& set = g_sets[set_index(ord)];
  set.models = std::move(ms);
  set.nout = n;
  set.tried_default = true;
  return TT_OK;
}

TT_EXPORT int32_t tt_selector_models(void) { return tt_selector_models_for_order(3); }

TT_EXPORT int32_t tt_selector_models_for_order(int32_t order) {
  const int si = set_index(order);
  if (si < 0) return 0;
  int n = 0;
  model_for(0, order, n);  // triggers the default load
  std::lock_guard<std::mutex> lk(g_mu);
  return (int32_t)g_sets[si].models.size();
}

TT_EXPORT tt_status tt_selector_scores(const taco_tensor_t* B, int32_t rank, tt_precision prec, float* scores,
                                       int32_t n) {
  clear_error();
  if (!B || !scores || n < 0) return set_error(TT_ERR_INVALID_ARGUMENT, "null argument");
  if (rank < 1 || rank > TT_MAX_RANK) return set_error(TT_ERR_INVALID_ARGUMENT, "rank %d", rank);
  CsfView v;
  tt_status s = csf_view(B, &v);
  if (s != TT_OK) return s;
  std::vector<float> sc;
  s = scores_for(B, v.order, rank, (int)prec, sc);
  if (s != TT_OK) return s;
  for (int i = 0; i < n; i++) scores[i] = i < (int)sc.size() ? sc[(size_t)i] : std::numeric_limits<float>::infinity();
  return TT_OK;
}
