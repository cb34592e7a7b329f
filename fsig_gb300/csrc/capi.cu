// C ABI of libfsig (include/fsig.h).
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "engine.h"
#include "match.h"
#include "mpnn.h"
#include "reader.h"

namespace fsig {

namespace {
thread_local std::string t_err;
}

int fail_cuda(cudaError_t e, const char* what, const char* file, int line) {
  t_err = std::string(cudaGetErrorString(e)) + " in " + what + " (" + file + ":" + std::to_string(line) + ")";
  return FSIG_ECUDA;
}
int fail(int status, const std::string& msg) {
  t_err = msg;
  return status;
}
const std::string& thread_error() { return t_err; }
void clear_thread_error() { t_err.clear(); }

}  // namespace fsig

using fsig::Engine;

struct fsig_graph_file {
  fsig::TveGraph g;
};

struct fsig_engine {
  Engine e;
};

namespace {

int finish(fsig_engine* h, int rc) {
  if (rc != FSIG_OK && h) h->e.last_error = fsig::thread_error();
  return rc;
}

int select(fsig_engine* h) {
  if (!h) return FSIG_EINVAL;
  cudaError_t err = cudaSetDevice(h->e.device);
  if (err != cudaSuccess) return fsig::fail_cuda(err, "cudaSetDevice", __FILE__, __LINE__);
  fsig::clear_thread_error();
  return FSIG_OK;
}

void fill_result(const fsig::HostQuery& hq, const fsig::BatchOutput& o, uint32_t qi, uint32_t g0, fsig_result* r) {
  const bool over = o.res[qi].aborted != 0;
  r->count = over ? 0 : o.res[qi].count;
  r->hash = over ? 0 : o.res[qi].hash;
  r->status = over ? FSIG_ELIMIT : FSIG_OK;
  r->num_vertices = hq.n;
  for (uint32_t i = 0; i < FSIG_MAX_QUERY; i++) {
    r->order[i] = i < hq.n ? o.orders[size_t(qi) * FSIG_MAX_QUERY + i] : 0;
    r->candidates[i] = i < hq.n ? o.counts[g0 + i] : 0;
    r->level_counts[i] = i < hq.n ? o.res[qi].levels[i] : 0;
  }
  r->ms_filter = o.ms_filter;
  r->ms_join = o.ms_join;
  r->work = o.res[qi].work;
}

void algo_options(int algo, int refine_iters, fsig::BatchOptions& o) {
  if (algo == FSIG_ALGO_FSIG) {
    o.filter_mode = fsig::kFilterDegree;
    o.refine_iters = refine_iters >= 0 ? refine_iters : 3;
    o.order_mode = fsig::kOrderMMatch;
  } else if (algo == FSIG_ALGO_GSI) {
    o.filter_mode = fsig::kFilterSignature;
    o.refine_iters = refine_iters >= 0 ? refine_iters : 0;
    o.order_mode = fsig::kOrderGSI;
  } else {
    o.filter_mode = fsig::kFilterDegree | fsig::kFilterSignature;
    o.refine_iters = refine_iters >= 0 ? refine_iters : 0;
    o.order_mode = fsig::kOrderGSI;
  }
}

}  // namespace

extern "C" {

const char* fsig_status_string(int s) {
  switch (s) {
    case FSIG_OK: return "ok";
    case FSIG_EINVAL: return "invalid argument";
    case FSIG_ENODEV: return "no usable CUDA device";
    case FSIG_ECUDA: return "CUDA error";
    case FSIG_EADMISSION: return "request does not fit the device arena";
    case FSIG_ENOGRAPH: return "no data graph loaded";
    case FSIG_EQUERY: return "invalid query";
    case FSIG_EIO: return "file error";
    case FSIG_ETIMEOUT: return "device wait timed out";
    case FSIG_EOVERFLOW: return "device work queue overflow";
    case FSIG_ELIMIT: return "query exceeded its work limit";
    default: return "unknown status";
  }
}

const char* fsig_last_error(const fsig_engine* h) {
  if (!h) return fsig::thread_error().c_str();
  return h->e.last_error.c_str();
}

int fsig_create(int device, uint64_t arena_bytes, fsig_engine** out) {
  if (!out) return FSIG_EINVAL;
  *out = nullptr;
  fsig::clear_thread_error();
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= device || device < 0) {
    fsig::fail(FSIG_ENODEV, "no CUDA device with this index");
    return FSIG_ENODEV;
  }
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return FSIG_ENODEV;
  if (prop.major != 10 || prop.minor != 3) {
    fsig::fail(FSIG_ENODEV, std::string("libfsig is built for sm_103 only; device is ") + prop.name);
    return FSIG_ENODEV;
  }
  auto* h = new (std::nothrow) fsig_engine();
  if (!h) return FSIG_EINVAL;
  Engine& e = h->e;
  e.device = device;
  e.num_sms = prop.multiProcessorCount;
  auto bail = [&](int code) {
    h->e.last_error = fsig::thread_error();
    if (e.arena.base) cudaFree(e.arena.base);
    if (e.stream) cudaStreamDestroy(e.stream);
    delete h;
    return code;
  };
  cudaError_t err = cudaSetDevice(device);
  if (err != cudaSuccess) return bail(fsig::fail_cuda(err, "cudaSetDevice", __FILE__, __LINE__));
  err = cudaStreamCreateWithFlags(&e.stream, cudaStreamNonBlocking);
  if (err != cudaSuccess) return bail(fsig::fail_cuda(err, "cudaStreamCreate", __FILE__, __LINE__));
  for (auto& ev : e.ev) {
    err = cudaEventCreate(&ev);
    if (err != cudaSuccess) return bail(fsig::fail_cuda(err, "cudaEventCreate", __FILE__, __LINE__));
  }
  for (auto& ev : e.ev_enum) {
    err = cudaEventCreate(&ev);
    if (err != cudaSuccess) return bail(fsig::fail_cuda(err, "cudaEventCreate", __FILE__, __LINE__));
  }
  for (auto& ev : e.ev_outer) {
    err = cudaEventCreate(&ev);
    if (err != cudaSuccess) return bail(fsig::fail_cuda(err, "cudaEventCreate", __FILE__, __LINE__));
  }
  uint64_t bytes = arena_bytes ? arena_bytes : uint64_t(prop.totalGlobalMem) / 4;
  err = cudaMalloc(&e.arena.base, bytes);
  if (err != cudaSuccess) return bail(fsig::fail(FSIG_EADMISSION, "cannot reserve the device arena"));
  e.arena.cap = bytes;
  *out = h;
  return FSIG_OK;
}

int fsig_destroy(fsig_engine* h) {
  if (!h) return FSIG_EINVAL;
  cudaSetDevice(h->e.device);
  if (h->e.stream) cudaStreamSynchronize(h->e.stream);
  for (auto& ev : h->e.ev)
    if (ev) cudaEventDestroy(ev);
  for (auto& ev : h->e.ev_enum)
    if (ev) cudaEventDestroy(ev);
  for (auto& ev : h->e.ev_outer)
    if (ev) cudaEventDestroy(ev);
  fsig::mpnn_free(h->e);
  if (h->e.gexec) cudaGraphExecDestroy(h->e.gexec);
  if (h->e.arena.base) cudaFree(h->e.arena.base);
  if (h->e.pinned) cudaFreeHost(h->e.pinned);
  if (h->e.stream) cudaStreamDestroy(h->e.stream);
  delete h;
  return FSIG_OK;
}

int fsig_load_graph(fsig_engine* h, uint32_t V, const int32_t* labels, uint64_t E, const uint32_t* edges) {
  int rc = select(h);
  if (rc) return finish(h, rc);
  if (!labels || (E && !edges)) return finish(h, fsig::fail(FSIG_EINVAL, "graph arrays missing"));
  return finish(h, fsig::build_device_graph(h->e, V, labels, E, edges));
}

int fsig_load_graph_file(fsig_engine* h, const char* path, int is_labeled) {
  int rc = select(h);
  if (rc) return finish(h, rc);
  if (!path) return finish(h, fsig::fail(FSIG_EINVAL, "no path"));
  fsig::TveGraph g;
  std::string err;
  if (fsig::read_tve(path, is_labeled, g, err) != 0) return finish(h, fsig::fail(FSIG_EIO, err));
  for (uint32_t v = 0; v < g.num_vertices; v++)
    if (g.labels[v] < 0) return finish(h, fsig::fail(FSIG_EIO, "vertex " + std::to_string(v) + " has no v record"));
  for (uint32_t x : g.edges)
    if (x >= g.num_vertices) return finish(h, fsig::fail(FSIG_EIO, "edge endpoint without a v record"));
  return finish(h, fsig::build_device_graph(h->e, g.num_vertices, g.labels.data(), g.edges.size() / 2,
                                            g.edges.data()));
}

int fsig_save_graph_cache(fsig_engine* h, const char* path) {
  int rc = select(h);
  if (rc) return finish(h, rc);
  if (!path) return finish(h, fsig::fail(FSIG_EINVAL, "no path"));
  return finish(h, fsig::save_graph_cache(h->e, path));
}

int fsig_load_graph_cache(fsig_engine* h, const char* path) {
  int rc = select(h);
  if (rc) return finish(h, rc);
  if (!path) return finish(h, fsig::fail(FSIG_EINVAL, "no path"));
  return finish(h, fsig::load_graph_cache(h->e, path));
}

int fsig_graph_info(const fsig_engine* h, uint32_t* V, uint64_t* nadj, int32_t* L, uint32_t* maxdeg) {
  if (!h) return FSIG_EINVAL;
  if (!h->e.has_graph) return FSIG_ENOGRAPH;
  if (V) *V = h->e.g.V;
  if (nadj) *nadj = h->e.g.nadj;
  if (L) *L = h->e.g.L;
  if (maxdeg) *maxdeg = h->e.g.max_deg;
  return FSIG_OK;
}

int fsig_set_segment_index(fsig_engine* h, int mode) {
  if (!h) return FSIG_EINVAL;
  if (mode != FSIG_SEGMENTS_AUTO && mode != FSIG_SEGMENTS_TABLE && mode != FSIG_SEGMENTS_ROWS)
    return finish(h, fsig::fail(FSIG_EINVAL, "unknown segment index"));
  h->e.seg_index = mode;
  return FSIG_OK;
}

int fsig_graph_layout(const fsig_engine* h, int* segment_index, uint64_t* bytes) {
  if (!h) return FSIG_EINVAL;
  if (!h->e.has_graph) return FSIG_ENOGRAPH;
  if (segment_index) *segment_index = h->e.g.lseg ? FSIG_SEGMENTS_TABLE : FSIG_SEGMENTS_ROWS;
  if (bytes) *bytes = fsig::store_bytes(h->e.g);
  return FSIG_OK;
}

int fsig_match(fsig_engine* h, const fsig_query* q, int algo, fsig_result* out) {
  int rc = select(h);
  if (rc) return finish(h, rc);
  if (!q || !out) return finish(h, fsig::fail(FSIG_EINVAL, "null argument"));
  if (algo != FSIG_ALGO_FSIG && algo != FSIG_ALGO_GSI && algo != FSIG_ALGO_FUSED)
    return finish(h, fsig::fail(FSIG_EINVAL, "unknown algorithm"));
  std::memset(out, 0, sizeof(*out));
  std::vector<fsig::HostQuery> qs(1);
  rc = fsig::prepare_query(*q, h->e.has_graph ? h->e.g.L : 0, qs[0]);
  if (rc) { out->status = rc; return finish(h, rc); }
  fsig::BatchOptions o;
  algo_options(algo, -1, o);
  if (!qs[0].has_given) o.host_order = algo == FSIG_ALGO_FSIG ? fsig::mmatch_order_host : fsig::gsi_order_host;
  else o.order_mode = fsig::kOrderGiven;
  fsig::BatchOutput bo;
  rc = fsig::run_batch(h->e, qs, o, bo);
  if (rc) { out->status = rc; return finish(h, rc); }
  fill_result(qs[0], bo, 0, 0, out);
  return FSIG_OK;
}

int fsig_match_range(fsig_engine* h, const fsig_query* q, int algo, uint32_t split_len, uint32_t task_begin,
                     uint32_t task_end, fsig_result* out, uint32_t* tasks_total) {
  int rc = select(h);
  if (rc) return finish(h, rc);
  if (!q || !out) return finish(h, fsig::fail(FSIG_EINVAL, "null argument"));
  if (algo != FSIG_ALGO_FSIG && algo != FSIG_ALGO_GSI && algo != FSIG_ALGO_FUSED)
    return finish(h, fsig::fail(FSIG_EINVAL, "unknown algorithm"));
  if (task_begin > task_end) return finish(h, fsig::fail(FSIG_EINVAL, "task_begin > task_end"));
  std::memset(out, 0, sizeof(*out));
  std::vector<fsig::HostQuery> qs(1);
  rc = fsig::prepare_query(*q, h->e.has_graph ? h->e.g.L : 0, qs[0]);
  if (rc) { out->status = rc; return finish(h, rc); }
  fsig::BatchOptions o;
  algo_options(algo, -1, o);
  if (!qs[0].has_given) o.host_order = algo == FSIG_ALGO_FSIG ? fsig::mmatch_order_host : fsig::gsi_order_host;
  else o.order_mode = fsig::kOrderGiven;
  o.split = split_len ? std::max<uint32_t>(split_len, 32u) : 256u;
  o.task_begin = task_begin;
  o.task_end = task_end;
  o.want_tasks = true;
  fsig::BatchOutput bo;
  rc = fsig::run_batch(h->e, qs, o, bo);
  if (rc) { out->status = rc; return finish(h, rc); }
  fill_result(qs[0], bo, 0, 0, out);
  if (tasks_total) *tasks_total = bo.tasks_total;
  return FSIG_OK;
}

int fsig_read_graph_file(const char* path, int is_labeled, fsig_graph_file** out) {
  return fsig_read_graph_file_threads(path, is_labeled, 0, out);
}

int fsig_read_graph_file_threads(const char* path, int is_labeled, uint64_t parallel_min_bytes, fsig_graph_file** out) {
  fsig::clear_thread_error();
  if (!path || !out) return FSIG_EINVAL;
  *out = nullptr;
  auto* f = new (std::nothrow) fsig_graph_file();
  if (!f) return FSIG_EINVAL;
  std::string err;
  if (fsig::read_tve(path, is_labeled, f->g, err, parallel_min_bytes) != 0) {
    delete f;
    fsig::fail(FSIG_EIO, err);
    return FSIG_EIO;
  }
  *out = f;
  return FSIG_OK;
}

int fsig_graph_file_data(const fsig_graph_file* f, uint32_t* V, const int32_t** labels, uint64_t* E,
                         const uint32_t** edges) {
  if (!f) return FSIG_EINVAL;
  if (V) *V = f->g.num_vertices;
  if (labels) *labels = f->g.labels.data();
  if (E) *E = f->g.edges.size() / 2;
  if (edges) *edges = f->g.edges.data();
  return FSIG_OK;
}

void fsig_free_graph_file(fsig_graph_file* f) { delete f; }

int fsig_match_embeddings(fsig_engine* h, const fsig_query* q, int algo, uint64_t buffer_rows,
                          fsig_embedding_sink sink, void* user, fsig_result* out) {
  int rc = select(h);
  if (rc) return finish(h, rc);
  if (!q || !out || !sink) return finish(h, fsig::fail(FSIG_EINVAL, "null argument"));
  if (algo != FSIG_ALGO_FSIG && algo != FSIG_ALGO_GSI && algo != FSIG_ALGO_FUSED)
    return finish(h, fsig::fail(FSIG_EINVAL, "unknown algorithm"));
  std::memset(out, 0, sizeof(*out));
  fsig::HostQuery hq;
  rc = fsig::prepare_query(*q, h->e.has_graph ? h->e.g.L : 0, hq);
  if (rc) { out->status = rc; return finish(h, rc); }
  fsig::BatchOptions o;
  algo_options(algo, -1, o);
  if (!hq.has_given) o.host_order = algo == FSIG_ALGO_FSIG ? fsig::mmatch_order_host : fsig::gsi_order_host;
  else o.order_mode = fsig::kOrderGiven;
  fsig::BatchOutput bo;
  rc = fsig::run_embeddings(h->e, hq, o, buffer_rows ? buffer_rows : (1ull << 20), sink, user, bo);
  if (rc) { out->status = rc; return finish(h, rc); }
  fill_result(hq, bo, 0, 0, out);
  return FSIG_OK;
}

namespace {
struct TextSink {
  FILE* fp;
  std::vector<char> buf;
  bool failed = false;
};

int text_sink(void* user, const uint32_t* rows, uint64_t num_rows, uint32_t width) {
  auto* t = static_cast<TextSink*>(user);
  t->buf.clear();
  t->buf.reserve(num_rows * width * 11);
  char tmp[12];
  for (uint64_t r = 0; r < num_rows; r++) {
    for (uint32_t c = 0; c < width; c++) {
      uint32_t v = rows[r * width + c];
      int k = 0;
      do { tmp[k++] = char('0' + v % 10); v /= 10; } while (v);
      while (k) t->buf.push_back(tmp[--k]);
      t->buf.push_back(c + 1 == width ? '\n' : ' ');
    }
  }
  if (std::fwrite(t->buf.data(), 1, t->buf.size(), t->fp) != t->buf.size()) {
    t->failed = true;
    return 1;
  }
  return 0;
}
}  // namespace

int fsig_write_embeddings(fsig_engine* h, const fsig_query* q, int algo, const char* path, fsig_result* out) {
  if (!h) return FSIG_EINVAL;
  if (!path) return finish(h, fsig::fail(FSIG_EINVAL, "no path"));
  TextSink t;
  t.fp = std::fopen(path, "wb");
  if (!t.fp) return finish(h, fsig::fail(FSIG_EIO, std::string("cannot open ") + path));
  int rc = fsig_match_embeddings(h, q, algo, 0, text_sink, &t, out);
  if (std::fclose(t.fp) != 0) t.failed = true;
  if (rc) return rc;
  if (t.failed) return finish(h, fsig::fail(FSIG_EIO, std::string("cannot write ") + path));
  return FSIG_OK;
}

int fsig_match_batch(fsig_engine* h, uint32_t nq, const fsig_query* qs, const fsig_batch_opts* opts,
                     fsig_result* out) {
  int rc = select(h);
  if (rc) return finish(h, rc);
  if ((nq && (!qs || !out))) return finish(h, fsig::fail(FSIG_EINVAL, "null argument"));
  fsig_batch_opts def{FSIG_ALGO_FUSED, FSIG_ORDER_HEURISTIC, -1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  const fsig_batch_opts& bo = opts ? *opts : def;
  if (bo.algo != FSIG_ALGO_FSIG && bo.algo != FSIG_ALGO_GSI && bo.algo != FSIG_ALGO_FUSED)
    return finish(h, fsig::fail(FSIG_EINVAL, "unknown algorithm"));
  std::vector<fsig::HostQuery> hq;
  std::vector<uint32_t> idx;
  hq.reserve(nq);
  for (uint32_t i = 0; i < nq; i++) {
    std::memset(&out[i], 0, sizeof(fsig_result));
    fsig::HostQuery x;
    int r = fsig::prepare_query(qs[i], h->e.has_graph ? h->e.g.L : 0, x);
    if (r) { out[i].status = r; continue; }
    if (bo.order_source == FSIG_ORDER_GIVEN && !x.has_given) { out[i].status = FSIG_EQUERY; continue; }
    hq.push_back(std::move(x));
    idx.push_back(i);
  }
  fsig::BatchOptions o;
  algo_options(bo.algo, bo.refine_iters, o);
  if (bo.order_source == FSIG_ORDER_GIVEN) o.order_mode = fsig::kOrderGiven;
  else if (bo.order_source == FSIG_ORDER_LEARNED) {
    if (!h->e.mpnn || !h->e.mpnn->loaded) return finish(h, fsig::fail(FSIG_EINVAL, "no order network loaded"));
    o.learned = true;
  }
  o.use_graph = bo.use_graph != 0;
  o.classes = bo.no_classes == 0;
  if (bo.learned_window) o.learned_window = bo.learned_window;
  if (bo.learned_prefix) o.learned_prefix = std::min<uint32_t>(bo.learned_prefix, 32u);
  if (bo.warps_per_block) {
    if (bo.warps_per_block > fsig::kEnumWarps) return finish(h, fsig::fail(FSIG_EINVAL, "warps_per_block too large"));
    o.warps_per_block = bo.warps_per_block;
  }
  if (bo.chunk) o.chunk = bo.chunk;
  if (bo.split_len) o.split = bo.split_len;
  if (bo.split_cycles) o.budget_cycles = (long long)bo.split_cycles;
  o.max_work = bo.max_work;
  if (bo.isect > 3) return finish(h, fsig::fail(FSIG_EINVAL, "unknown intersection strategy"));
  o.isect = bo.isect;
  if (bo.refine_coop) o.refine_coop = bo.refine_coop;
  fsig::BatchOutput out_b;
  rc = fsig::run_batch(h->e, hq, o, out_b);
  if (rc) return finish(h, rc);
  uint32_t g0 = 0;
  for (size_t k = 0; k < hq.size(); k++) {
    fill_result(hq[k], out_b, uint32_t(k), g0, &out[idx[k]]);
    g0 += hq[k].n;
  }
  return FSIG_OK;
}

uint32_t fsig_mpnn_param_count(void) { return uint32_t(fsig::kParams); }

int fsig_mpnn_set_params(fsig_engine* h, const float* params, uint32_t count) {
  int rc = select(h);
  if (rc) return finish(h, rc);
  if (!params || count != uint32_t(fsig::kParams)) return finish(h, fsig::fail(FSIG_EINVAL, "parameter count"));
  return finish(h, fsig::mpnn_set_params(h->e, params));
}

int fsig_mpnn_get_params(fsig_engine* h, float* params, uint32_t count) {
  int rc = select(h);
  if (rc) return finish(h, rc);
  if (!params || count != uint32_t(fsig::kParams)) return finish(h, fsig::fail(FSIG_EINVAL, "parameter count"));
  return finish(h, fsig::mpnn_get_params(h->e, params));
}

int fsig_mpnn_features(fsig_engine* h, uint32_t nq, const fsig_query* qs, int algo, const uint32_t* cand,
                       float* features) {
  int rc = select(h);
  if (rc) return finish(h, rc);
  if (nq && (!qs || !cand || !features)) return finish(h, fsig::fail(FSIG_EINVAL, "null argument"));
  std::vector<fsig::HostQuery> hq(nq);
  for (uint32_t i = 0; i < nq; i++) {
    rc = fsig::prepare_query(qs[i], h->e.has_graph ? h->e.g.L : 0, hq[i]);
    if (rc) return finish(h, rc);
  }
  fsig::BatchOptions o;
  algo_options(algo, -1, o);
  return finish(h, fsig::run_features(h->e, hq, cand, o.order_mode, features));
}

int fsig_mpnn_forward(fsig_engine* h, uint32_t ng, const uint32_t* goff, const float* feat, const uint32_t* nbr,
                      float* scores) {
  int rc = select(h);
  if (rc) return finish(h, rc);
  if (!goff || (goff[ng] && (!feat || !nbr || !scores))) return finish(h, fsig::fail(FSIG_EINVAL, "null argument"));
  return finish(h, fsig::mpnn_run(h->e, ng, goff, feat, nbr, nullptr, 0.f, scores, nullptr, nullptr));
}

int fsig_mpnn_train_step(fsig_engine* h, uint32_t ng, const uint32_t* goff, const float* feat, const uint32_t* nbr,
                         const float* targets, float lr, float* loss, float* grads) {
  int rc = select(h);
  if (rc) return finish(h, rc);
  if (!goff || !targets || (goff[ng] && (!feat || !nbr))) return finish(h, fsig::fail(FSIG_EINVAL, "null argument"));
  return finish(h, fsig::mpnn_run(h->e, ng, goff, feat, nbr, targets, lr, nullptr, loss, grads));
}

int fsig_last_stats(const fsig_engine* h, fsig_batch_stats* out) {
  if (!h || !out) return FSIG_EINVAL;
  *out = h->e.last;
  return FSIG_OK;
}

int fsig_set_queue_waits(fsig_engine* h, uint64_t ready_wait_ns, uint64_t idle_wait_ns, int unpublished) {
  if (!h) return FSIG_EINVAL;
  constexpr uint64_t kMaxWaitNs = 60ull * 1000000000ull;
  if (ready_wait_ns > kMaxWaitNs || idle_wait_ns > kMaxWaitNs || (unpublished != 0 && unpublished != 1))
    return FSIG_EINVAL;
  h->e.ready_wait_ns = ready_wait_ns ? ready_wait_ns : 200000000ull;
  h->e.idle_wait_ns = idle_wait_ns ? idle_wait_ns : 2000000000ull;
  h->e.inject_unpublished = uint32_t(unpublished);
  return FSIG_OK;
}

int fsig_plan_order(const fsig_query* q, int algo, const uint32_t* cand, uint32_t* order, uint32_t* types,
                    uint32_t* classes) {
  fsig::clear_thread_error();
  if (!q || !cand || !order) return FSIG_EINVAL;
  fsig::HostQuery hq;
  int rc = fsig::prepare_query(*q, 0, hq);
  if (rc) return rc;
  if (algo == FSIG_ALGO_FSIG) {
    fsig::mmatch_order_host(hq, cand, order);
    fsig::mmatch_structure(hq, types, classes);
  } else if (algo == FSIG_ALGO_GSI || algo == FSIG_ALGO_FUSED) {
    fsig::gsi_order_host(hq, cand, order);
  } else {
    return FSIG_EINVAL;
  }
  return FSIG_OK;
}

int fsig_build_csr(fsig_engine* h, uint32_t V, uint64_t E, const uint32_t* edges, uint32_t* offsets, uint32_t* adj) {
  int rc = select(h);
  if (rc) return finish(h, rc);
  if (!offsets || (E && (!edges || !adj))) return finish(h, fsig::fail(FSIG_EINVAL, "null argument"));
  return finish(h, fsig::build_reference_csr(h->e, V, E, edges, offsets, adj));
}

int fsig_build_signature(fsig_engine* h, uint32_t V, const int32_t* labels, const uint32_t* offsets,
                         const uint32_t* adj, int column_oriented, uint32_t* signature) {
  int rc = select(h);
  if (rc) return finish(h, rc);
  if (!labels || !offsets || !signature) return finish(h, fsig::fail(FSIG_EINVAL, "null argument"));
  return finish(h, fsig::build_reference_signature(h->e, V, labels, offsets, adj, column_oriented, signature));
}

int fsig_build_pcsr(fsig_engine* h, uint32_t V, int32_t L, const int32_t* labels, const uint32_t* offsets,
                    const uint32_t* adj, uint32_t* unit_keys, uint32_t* unit_edges, uint32_t* table,
                    uint32_t* edges) {
  int rc = select(h);
  if (rc) return finish(h, rc);
  if (!labels || !offsets || !unit_keys || !unit_edges || (offsets[V] && !adj))
    return finish(h, fsig::fail(FSIG_EINVAL, "null argument"));
  return finish(h, fsig::build_reference_pcsr(h->e, V, L, labels, offsets, adj, unit_keys, unit_edges, table, edges));
}

int fsig_filter_classes(fsig_engine* h, const fsig_query* q, int algo, int refine_iters, int classes,
                        uint8_t* flags) {
  int rc = select(h);
  if (rc) return finish(h, rc);
  if (!q || !flags) return finish(h, fsig::fail(FSIG_EINVAL, "null argument"));
  fsig::HostQuery hq;
  rc = fsig::prepare_query(*q, h->e.has_graph ? h->e.g.L : 0, hq);
  if (rc) return finish(h, rc);
  fsig::BatchOptions o;
  algo_options(algo, refine_iters, o);
  return finish(h, fsig::run_filter_probe(h->e, hq, o.filter_mode, o.refine_iters, classes != 0, flags));
}

int fsig_filter(fsig_engine* h, const fsig_query* q, int algo, int refine_iters, uint8_t* flags) {
  return fsig_filter_classes(h, q, algo, refine_iters, 1, flags);
}

int fsig_refine_classes(const fsig_query* q, uint32_t* classes, uint32_t* dominated) {
  fsig::clear_thread_error();
  if (!q) return FSIG_EINVAL;
  fsig::HostQuery hq;
  int rc = fsig::prepare_query(*q, 0, hq);
  if (rc) return rc;
  uint8_t c[fsig::kMaxQ], d[fsig::kMaxQ];
  fsig::refine_classes(hq, c, d);
  for (uint32_t u = 0; u < hq.n; u++) {
    if (classes) classes[u] = c[u];
    if (dominated) dominated[u] = d[u];
  }
  return FSIG_OK;
}

// Allocation-free filter: the arena is not touched; see run_filter_noalloc.
int fsig_filter_noalloc(fsig_engine* h, const fsig_query* q, int algo, uint8_t* d_flags) {
  int rc = select(h);
  if (rc) return finish(h, rc);
  if (!q || !d_flags) return finish(h, fsig::fail(FSIG_EINVAL, "null argument"));
  if (algo != FSIG_ALGO_FSIG && algo != FSIG_ALGO_GSI && algo != FSIG_ALGO_FUSED)
    return finish(h, fsig::fail(FSIG_EINVAL, "unknown algorithm"));
  fsig::BatchOptions o;
  algo_options(algo, 0, o);
  return finish(h, fsig::run_filter_noalloc(h->e, *q, o.filter_mode, d_flags));
}

}  // extern "C"
