// api.cu -- the C ABI of libbeastgpu (include/beastgpu.h): handles, uploads, the chunked
// assembly driver, dense solves, GMRES and the one-call solve job.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "internal.h"

static cudaEvent_t ev_get(beast_ctx* c) {
  if (!c->evpool.empty()) {
    cudaEvent_t e = c->evpool.back();
    c->evpool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

bool ctx_lookahead_streams(beast_ctx* ctx) {
  if (ctx->aux) return true;
  int lo = 0, hi = 0;
  if (cudaDeviceGetStreamPriorityRange(&lo, &hi) != cudaSuccess) hi = 0;
  cudaStream_t s = nullptr;
  if (cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, hi) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  for (auto& e : ctx->la_ev)
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
      cudaGetLastError();
      for (auto& f : ctx->la_ev)
        if (f) cudaEventDestroy(f), f = nullptr;
      cudaStreamDestroy(s);
      return false;
    }
  ctx->aux = s;
  return true;
}

ProfScope::ProfScope(beast_ctx* c, int k, double w, int nlaunch) : ctx(c), kind(k), work(w) {
  ctx->launches += nlaunch;
  if (ctx->prof_on && ((ctx->prof_mask >> kind) & 1u)) {
    a = ev_get(ctx);
    cudaEventRecord(a, ctx->stream);
  }
}
ProfScope::~ProfScope() {
  if (!a) return;
  cudaEvent_t b = ev_get(ctx);
  cudaEventRecord(b, ctx->stream);
  ctx->prof.push_back(ProfRec{kind, a, b, work});
}

int beast_fail(beast_ctx* ctx, int code, const std::string& msg) {
  if (ctx) ctx->err = msg;
  return code;
}

#define ARG_CHECK(ctx, cond, msg) \
  do {                            \
    if (!(cond)) return beast_fail((ctx), BEAST_ERR_ARG, (msg)); \
  } while (0)

namespace {

// device workspace: grows on demand, kept by the context
int ws_reserve(beast_ctx* ctx, size_t bytes) {
  if (bytes <= ctx->ws_size) return BEAST_OK;
  if (ctx->ws) {
    cudaStreamSynchronize(ctx->stream);
    cudaFree(ctx->ws);
    ctx->ws = nullptr;
    ctx->ws_size = 0;
  }
  cudaError_t e = cudaMalloc(&ctx->ws, bytes);
  if (e != cudaSuccess) {
    ctx->ws = nullptr;
    return beast_fail(ctx, BEAST_ERR_OOM, "workspace allocation of " + std::to_string(bytes) +
                                              " bytes failed: " + cudaGetErrorString(e));
  }
  ctx->ws_size = bytes;
  return BEAST_OK;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

OpParams to_params(const beast_op_desc* op) {
  OpParams p;
  p.kind = op->kind;
  p.gr = op->gamma_re;
  p.gi = op->gamma_im;
  p.ar = op->alpha_re;
  p.ai = op->alpha_im;
  p.br = op->beta_re;
  p.bi = op->beta_im;
  return p;
}

int set_device(beast_ctx* ctx) {
  BEAST_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  return BEAST_OK;
}

}  // namespace

extern "C" {

const char* beast_version(void) { return "beastgpu 0.1 (sm_103a)"; }

int beast_ctx_create(int device, beast_ctx** out) {
  if (!out) return BEAST_ERR_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return BEAST_ERR_CUDA;
  if (device < 0 || device >= ndev) return BEAST_ERR_ARG;
  beast_ctx* c = new beast_ctx();
  c->device = device;
  if (cudaSetDevice(device) != cudaSuccess) {
    delete c;
    return BEAST_ERR_CUDA;
  }
  cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
  // workspace (factor copies, Zcell chunks, tensor-core operands) is stream-ordered memory
  // of the device's default pool: keep what is freed in the pool instead of returning it at
  // every synchronisation, so that repeated solves do not map gigabytes again each time
  // (the pool is trimmed when the context is destroyed)
  {
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
      uint64_t keep = UINT64_MAX;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
  }
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return BEAST_ERR_CUDA;
  }
  c->own_stream = true;
  size_t fr = 0, tot = 0;
  cudaMemGetInfo(&fr, &tot);
  c->ws_limit = fr / 4;
  if (cudaMalloc(&c->d_flag, 64) != cudaSuccess) {
    cudaStreamDestroy(c->stream);
    delete c;
    return BEAST_ERR_OOM;
  }
  *out = c;
  return BEAST_OK;
}

int beast_ctx_destroy(beast_ctx* ctx) {
  if (!ctx) return BEAST_OK;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  if (ctx->aux) {
    cudaStreamSynchronize(ctx->aux);
    for (auto& e : ctx->la_ev)
      if (e) cudaEventDestroy(e);
    cudaStreamDestroy(ctx->aux);
  }
  if (ctx->ws) cudaFree(ctx->ws);
  if (ctx->d_flag) cudaFree(ctx->d_flag);
  for (auto& kv : ctx->ss_tabs) cudaFree(kv.second);
  for (auto& r : ctx->prof) {
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  for (auto e : ctx->evpool) cudaEventDestroy(e);
  if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, ctx->device) == cudaSuccess) cudaMemPoolTrimTo(pool, 0);
  delete ctx;
  return BEAST_OK;
}

int beast_last_error(beast_ctx* ctx, char* buf, size_t len) {
  if (!buf || len == 0) return BEAST_ERR_ARG;
  const char* m = ctx ? ctx->err.c_str() : "no context";
  snprintf(buf, len, "%s", m);
  return BEAST_OK;
}

int beast_ctx_set_stream(beast_ctx* ctx, void* stream) {
  ARG_CHECK(ctx, ctx, "null context");
  if (!stream) return BEAST_OK;
  cudaStreamSynchronize(ctx->stream);
  if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
  ctx->stream = (cudaStream_t)stream;
  ctx->own_stream = false;
  return BEAST_OK;
}

int beast_ctx_set_workspace_limit(beast_ctx* ctx, size_t bytes) {
  ARG_CHECK(ctx, ctx && bytes >= (1u << 20), "workspace limit below 1 MiB");
  ctx->ws_limit = bytes;
  return BEAST_OK;
}

int beast_prof_enable(beast_ctx* ctx, int on) {
  ARG_CHECK(ctx, ctx, "null context");
  cudaStreamSynchronize(ctx->stream);
  for (auto& r : ctx->prof) {
    ctx->evpool.push_back(r.a);
    ctx->evpool.push_back(r.b);
  }
  ctx->prof.clear();
  // events for the brackets to come, made here rather than at the first record of each: an
  // event creation costs the issuing thread several microseconds, which the bracketed
  // launches would otherwise wait for (about two thousand records per dense solve at n = 30720)
  constexpr size_t kEventsReady = 8192;
  while (on && ctx->evpool.size() < kEventsReady) {
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) {
      cudaGetLastError();
      break;
    }
    ctx->evpool.push_back(e);
  }
  ctx->prof_on = on != 0;
  ctx->prof_mask = 0xffffffffu;
  ctx->launches = 0;
  return BEAST_OK;
}

int beast_prof_enable_kinds(beast_ctx* ctx, unsigned int mask) {
  int rc = beast_prof_enable(ctx, mask != 0);
  if (rc == BEAST_OK) ctx->prof_mask = mask;
  return rc;
}

int beast_prof_read(beast_ctx* ctx, int kind, double* ms, int64_t* launches, double* work) {
  ARG_CHECK(ctx, ctx && kind >= 0 && kind < PK_COUNT, "bad profiler query");
  BEAST_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  double t = 0, w = 0;
  int64_t nl = 0;
  for (auto& r : ctx->prof) {
    if (r.kind != kind) continue;
    float e = 0;
    cudaEventElapsedTime(&e, r.a, r.b);
    t += e;
    w += r.work;
    ++nl;
  }
  if (ms) *ms = t;
  if (launches) *launches = nl;
  if (work) *work = w;
  return BEAST_OK;
}

int beast_last_factor_mode(beast_ctx* ctx, int* mode) {
  if (!ctx || !mode) return BEAST_ERR_ARG;
  *mode = ctx->last_factor_mode;
  return BEAST_OK;
}

int beast_prof_launches(beast_ctx* ctx, int64_t* n) {
  ARG_CHECK(ctx, ctx && n, "null argument");
  *n = ctx->launches;
  return BEAST_OK;
}

int beast_pool_stats(beast_ctx* ctx, size_t* reserved, size_t* reserved_high, size_t* used, size_t* used_high) {
  ARG_CHECK(ctx, ctx && reserved && reserved_high && used && used_high, "null argument");
  cudaMemPool_t pool;
  BEAST_CUDA_TRY(ctx, cudaDeviceGetDefaultMemPool(&pool, ctx->device));
  uint64_t v[4] = {0, 0, 0, 0};
  const cudaMemPoolAttr at[4] = {cudaMemPoolAttrReservedMemCurrent, cudaMemPoolAttrReservedMemHigh,
                                 cudaMemPoolAttrUsedMemCurrent, cudaMemPoolAttrUsedMemHigh};
  for (int k = 0; k < 4; ++k) BEAST_CUDA_TRY(ctx, cudaMemPoolGetAttribute(pool, at[k], &v[k]));
  *reserved = v[0];
  *reserved_high = v[1];
  *used = v[2];
  *used_high = v[3];
  return BEAST_OK;
}

int beast_ctx_set_wait_limit(beast_ctx* ctx, int64_t polls) {
  ARG_CHECK(ctx, ctx && polls >= 0, "invalid wait limit");
  ctx->trsv_spin_max = polls;
  return BEAST_OK;
}

int beast_ctx_synchronize(beast_ctx* ctx) {
  ARG_CHECK(ctx, ctx, "null context");
  BEAST_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return BEAST_OK;
}

int beast_mesh_upload(beast_ctx* ctx, const double* verts, int64_t nv, const int32_t* cells,
                      int64_t nc, int index_base, beast_mesh** out) {
  ARG_CHECK(ctx, ctx && out && verts && cells && nv > 0 && nc > 0, "invalid mesh arguments");
  ARG_CHECK(ctx, index_base == 0 || index_base == 1, "index_base must be 0 or 1");
  if (set_device(ctx)) return BEAST_ERR_CUDA;
  std::vector<int> c(3 * nc);
  for (int64_t i = 0; i < 3 * nc; ++i) {
    int v = cells[i] - index_base;
    ARG_CHECK(ctx, v >= 0 && v < nv, "cell vertex index out of range");
    c[i] = v;
  }
  beast_mesh* m = new beast_mesh();
  m->ctx = ctx;
  m->nv = nv;
  m->nc = nc;
  cudaError_t e = cudaMalloc(&m->verts, sizeof(double) * 3 * nv);
  if (e == cudaSuccess) e = cudaMalloc(&m->cells, sizeof(int) * 3 * nc);
  if (e == cudaSuccess) e = cudaMemcpyAsync(m->verts, verts, sizeof(double) * 3 * nv, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(m->cells, c.data(), sizeof(int) * 3 * nc, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    cudaFree(m->verts);
    cudaFree(m->cells);
    delete m;
    return beast_fail(ctx, BEAST_ERR_CUDA, std::string("mesh upload: ") + cudaGetErrorString(e));
  }
  *out = m;
  return BEAST_OK;
}

int beast_mesh_free(beast_mesh* m) {
  if (!m) return BEAST_OK;
  cudaSetDevice(m->ctx->device);
  cudaStreamSynchronize(m->ctx->stream);
  cudaFree(m->verts);
  cudaFree(m->cells);
  if (m->children) cudaFree(m->children);
  delete m;
  return BEAST_OK;
}

int beast_mesh_set_children(beast_ctx* ctx, beast_mesh* m, int nchild, const double* child_verts) {
  ARG_CHECK(ctx, ctx && m && child_verts, "null argument");
  ARG_CHECK(ctx, nchild >= 1 && nchild <= MAX_CHILDREN, "nchild must be in 1..8");
  ARG_CHECK(ctx, m->ctx == ctx, "the mesh belongs to another context");
  if (set_device(ctx)) return BEAST_ERR_CUDA;
  const size_t bytes = sizeof(double) * 9 * (size_t)nchild * (size_t)m->nc;
  double* d = nullptr;
  cudaError_t e = cudaMalloc(&d, bytes);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d, child_verts, bytes, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    if (d) cudaFree(d);
    return beast_fail(ctx, BEAST_ERR_CUDA, std::string("children upload: ") + cudaGetErrorString(e));
  }
  if (m->children) cudaFree(m->children);
  m->children = d;
  m->nchild = nchild;
  return BEAST_OK;
}

int beast_space_upload(beast_ctx* ctx, const beast_mesh* mesh, int kind, int64_t ncells,
                       const int64_t* cells, int maxfn, int nshapes, const int64_t* ad_dof,
                       const double* ad_coeff, int64_t nfuncs, int index_base, beast_space** out) {
  ARG_CHECK(ctx, ctx && mesh && out && cells && ad_dof && ad_coeff, "null argument");
  ARG_CHECK(ctx, kind == BEAST_P0 || kind == BEAST_P1 || kind == BEAST_RT, "unknown space kind");
  ARG_CHECK(ctx, nshapes == (kind == BEAST_P0 ? 1 : 3), "nshapes does not match the space kind");
  ARG_CHECK(ctx, ncells > 0 && maxfn >= 1 && nfuncs > 0 && nfuncs < (1LL << 31), "invalid sizes");
  ARG_CHECK(ctx, index_base == 0 || index_base == 1, "index_base must be 0 or 1");
  if (set_device(ctx)) return BEAST_ERR_CUDA;
  beast_space* s = new beast_space();
  s->ctx = ctx;
  s->mesh = mesh;
  s->kind = kind;
  s->nshapes = nshapes;
  s->maxfn = maxfn;
  s->ncells = ncells;
  s->nfuncs = nfuncs;
  std::vector<int> hc(ncells), c2a(mesh->nc, -1);
  for (int64_t c = 0; c < ncells; ++c) {
    int64_t mc = cells[c] - index_base;
    if (mc < 0 || mc >= mesh->nc) {
      delete s;
      return beast_fail(ctx, BEAST_ERR_ARG, "active cell index out of range");
    }
    hc[c] = (int)mc;
    c2a[mc] = (int)c;
  }
  const int64_t nad = ncells * nshapes * maxfn;
  s->h_ad_dof.resize(nad);
  s->h_ad_coeff.assign(ad_coeff, ad_coeff + nad);
  std::vector<int64_t> cnt(nfuncs + 1, 0);
  for (int64_t i = 0; i < nad; ++i) {
    int64_t d = ad_dof[i] - index_base;
    if (ad_dof[i] < index_base) d = -1;
    if (d >= nfuncs) {
      delete s;
      return beast_fail(ctx, BEAST_ERR_ARG, "assembly data dof index out of range");
    }
    s->h_ad_dof[i] = (int)d;
    if (d >= 0) cnt[d + 1]++;
  }
  for (int64_t f = 0; f < nfuncs; ++f) cnt[f + 1] += cnt[f];
  s->h_fn_ptr = cnt;
  s->h_fn_cell.resize(cnt[nfuncs]);
  s->h_fn_shape.resize(cnt[nfuncs]);
  s->h_fn_coeff.resize(cnt[nfuncs]);
  std::vector<int64_t> fill(cnt.begin(), cnt.end() - 1);
  for (int64_t c = 0; c < ncells; ++c)
    for (int r = 0; r < nshapes; ++r)
      for (int k = 0; k < maxfn; ++k) {
        int64_t i = (c * nshapes + r) * maxfn + k;
        int d = s->h_ad_dof[i];
        if (d < 0) continue;
        int64_t o = fill[d]++;
        s->h_fn_cell[o] = (int)c;
        s->h_fn_shape[o] = r;
        s->h_fn_coeff[o] = s->h_ad_coeff[i];
      }
  cudaStream_t st = ctx->stream;
  cudaError_t e = cudaSuccess;
  auto up = [&](void** dst, const void* src, size_t bytes) {
    if (e != cudaSuccess) return;
    e = cudaMalloc(dst, std::max<size_t>(bytes, 16));
    if (e == cudaSuccess && bytes) e = cudaMemcpyAsync(*dst, src, bytes, cudaMemcpyHostToDevice, st);
  };
  up((void**)&s->cells, hc.data(), sizeof(int) * ncells);
  up((void**)&s->cell2act, c2a.data(), sizeof(int) * mesh->nc);
  up((void**)&s->ad_dof, s->h_ad_dof.data(), sizeof(int) * nad);
  up((void**)&s->ad_coeff, s->h_ad_coeff.data(), sizeof(double) * nad);
  up((void**)&s->fn_ptr, s->h_fn_ptr.data(), sizeof(int64_t) * (nfuncs + 1));
  up((void**)&s->fn_cell, s->h_fn_cell.data(), sizeof(int) * s->h_fn_cell.size());
  up((void**)&s->fn_shape, s->h_fn_shape.data(), sizeof(int) * s->h_fn_shape.size());
  up((void**)&s->fn_coeff, s->h_fn_coeff.data(), sizeof(double) * s->h_fn_coeff.size());
  s->unit_coef = true;
  for (double c : s->h_fn_coeff) s->unit_coef = s->unit_coef && (c == 1.0 || c == -1.0);
  // Zcell row order on the test side: active cells by their first (lowest) function, so that
  // consecutive functions read nearby Zcell rows in the gather
  {
    std::vector<int64_t> key(ncells, INT64_MAX);
    for (int64_t f = 0; f < nfuncs; ++f)
      for (int64_t e = s->h_fn_ptr[f]; e < s->h_fn_ptr[f + 1]; ++e)
        key[s->h_fn_cell[e]] = std::min<int64_t>(key[s->h_fn_cell[e]], f);
    std::vector<int> perm(ncells), pos(ncells);
    for (int64_t c = 0; c < ncells; ++c) perm[c] = (int)c;
    std::stable_sort(perm.begin(), perm.end(), [&](int a, int b) { return key[a] < key[b]; });
    for (int64_t i = 0; i < ncells; ++i) pos[perm[i]] = (int)i;
    up((void**)&s->tperm, perm.data(), sizeof(int) * ncells);
    up((void**)&s->tpos, pos.data(), sizeof(int) * ncells);
    // the entry of each (active cell, shape), and by Zcell position for the far kernels
    s->h_cs2e.assign(ncells * nshapes, -1);
    s->injective = true;
    for (int64_t f = 0; f < (int64_t)s->h_fn_cell.size(); ++f) {
      int& slot = s->h_cs2e[(int64_t)s->h_fn_cell[f] * nshapes + s->h_fn_shape[f]];
      if (slot >= 0) s->injective = false;
      slot = (int)f;
    }
    if (s->injective) {
      std::vector<int> zr(ncells * nshapes);
      for (int64_t i = 0; i < ncells; ++i)
        for (int r = 0; r < nshapes; ++r) zr[i * nshapes + r] = s->h_cs2e[(int64_t)perm[i] * nshapes + r];
      up((void**)&s->zrow_entry, zr.data(), sizeof(int) * zr.size());
    }
  }
  if (e == cudaSuccess) e = cudaMalloc(&s->geo, sizeof(double) * GEO_STRIDE * ncells);
  if (e == cudaSuccess) e = cudaMalloc(&s->geof, sizeof(float) * 4 * ncells);
  if (e == cudaSuccess) e = launch_geometry(s, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    beast_space_free(s);
    return beast_fail(ctx, BEAST_ERR_CUDA, std::string("space upload: ") + cudaGetErrorString(e));
  }
  *out = s;
  return BEAST_OK;
}

int beast_space_free(beast_space* s) {
  if (!s) return BEAST_OK;
  cudaSetDevice(s->ctx->device);
  cudaStreamSynchronize(s->ctx->stream);
  void* ptrs[] = {s->cells, s->cell2act, s->ad_dof, s->ad_coeff, s->geo, s->geof,
                  s->fn_ptr, s->fn_cell, s->fn_shape, s->fn_coeff, s->tperm, s->tpos, s->zrow_entry};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  delete s;
  return BEAST_OK;
}

// ---------------------------------------------------------------------------------------
// assembly driver
// ---------------------------------------------------------------------------------------
static int assemble_device(beast_ctx* ctx, const beast_op_desc* op, const beast_qs_desc* qs,
                           const beast_space* ts, const beast_space* bs, int precision, void* Z,
                           int64_t ldz, int z_c64, int64_t row_off, int64_t col_off, double cr,
                           double ci, int accumulate) {
  cudaStream_t st = ctx->stream;
  const int nst = ts->kind == BEAST_P0 ? 1 : 3, nsb = bs->kind == BEAST_P0 ? 1 : 3;
  // cell-pair blocks laid out by function entries when both spaces allow it (the gather then
  // reads each function's rows and columns as contiguous runs); else by cells.
  // BEAST_ZCELL_LAYOUT=cell forces the cell layout.
  bool entry_layout = ts->injective && bs->injective;
  {
    const char* ev = getenv("BEAST_ZCELL_LAYOUT");
    if (ev && ev[0] == 'c') entry_layout = false;
  }
  const int64_t ldc = entry_layout ? ts->h_fn_ptr[ts->nfuncs] : (int64_t)nst * ts->ncells;
  const int zfmt = precision == BEAST_MIXED                                                  ? ZCELL_C64
                   : precision == BEAST_MIXED_ACCURATE || precision == BEAST_MIXED_BALANCED ? ZCELL_DF
                                                                                              : ZCELL_C128;
  const size_t elem = zfmt == ZCELL_C64 ? 8 : 16;
  // rules
  TriRuleDev ro, ri, ron, rin;
  ARG_CHECK(ctx, make_trirule(qs->outer_far, &ro) && make_trirule(qs->inner_far, &ri),
            "far rule degree not available (1..10)");
  // DoubleNumQStrat pairs that come close are evaluated by the near kernel too (class 4)
  const bool has_near = true;
  if (qs->kind == BEAST_QS_WILTON_SAUTER || qs->kind == BEAST_QS_TEST_REFINES_TRIAL ||
      qs->kind == BEAST_QS_TRIAL_REFINES_TEST) {
    ARG_CHECK(ctx, make_trirule(qs->outer_near, &ron) && make_trirule(qs->inner_near, &rin),
              "near rule degree not available (1..10)");
  } else {
    ron = ro;
    rin = ri;
  }
  if (qs->kind != BEAST_QS_DOUBLENUM)
    ARG_CHECK(ctx, qs->ss_face >= 1 && qs->ss_face <= 20 && qs->ss_edge >= 1 && qs->ss_edge <= 20 &&
                       qs->ss_vert >= 1 && qs->ss_vert <= 20,
              "Sauter-Schwab orders must be in 1..20");
  // chunking over trial dofs: cells needed per chunk fit the workspace
  const int64_t near_cap = std::max<int64_t>(1 << 16, 48 * ts->ncells);
  size_t fixed = align256(near_cap * sizeof(NearPair)) + align256(sizeof(int) * bs->ncells) * 2 + 4096;
  size_t budget = ctx->ws_limit > fixed ? ctx->ws_limit - fixed : 0;
  int64_t max_cells = (int64_t)(budget / ((size_t)ldc * nsb * elem));
  ARG_CHECK(ctx, max_cells >= 4, "workspace limit too small for one trial chunk");
  max_cells = std::min<int64_t>(max_cells, bs->ncells);
  std::vector<int> qlocal_h(bs->ncells, -1), qcells_h;
  qcells_h.reserve(max_cells);
  struct Chunk {
    int64_t n0, n1;
    std::vector<int> cells;
  };
  std::vector<Chunk> chunks;
  {
    int64_t n0 = 0;
    std::vector<int> cur;
    std::vector<char> in(bs->ncells, 0);
    for (int64_t n = 0; n < bs->nfuncs; ++n) {
      int add = 0;
      for (int64_t f = bs->h_fn_ptr[n]; f < bs->h_fn_ptr[n + 1]; ++f) add += !in[bs->h_fn_cell[f]];
      if ((int64_t)cur.size() + add > max_cells && n > n0) {
        chunks.push_back({n0, n, cur});
        for (int c : cur) in[c] = 0;
        cur.clear();
        n0 = n;
      }
      for (int64_t f = bs->h_fn_ptr[n]; f < bs->h_fn_ptr[n + 1]; ++f) {
        int c = bs->h_fn_cell[f];
        if (!in[c]) {
          in[c] = 1;
          cur.push_back(c);
        }
      }
    }
    chunks.push_back({n0, bs->nfuncs, cur});
  }
  int64_t maxq = 1;
  for (auto& c : chunks) maxq = std::max<int64_t>(maxq, (int64_t)c.cells.size());
  size_t zbytes = align256((size_t)ldc * nsb * maxq * elem);
  size_t need = zbytes + align256(near_cap * sizeof(NearPair)) + align256(sizeof(int) * maxq) +
                align256(sizeof(int) * bs->ncells) + 256 + align256(sizeof(int) * nsb * maxq);
  int rc = ws_reserve(ctx, need);
  if (rc) return rc;
  char* w = (char*)ctx->ws;
  void* zcell = w;
  NearPair* nearl = (NearPair*)(w + zbytes);
  int* qcells_d = (int*)((char*)nearl + align256(near_cap * sizeof(NearPair)));
  int* qlocal_d = (int*)((char*)qcells_d + align256(sizeof(int) * maxq));
  int* counter = (int*)((char*)qlocal_d + align256(sizeof(int) * bs->ncells));
  int* zcol_d = (int*)((char*)counter + 256);
  BEAST_CUDA_TRY(ctx, cudaMemsetAsync(ctx->d_flag, 0, 64, st));
  std::vector<int> ql(bs->ncells, -1), zcol_h;
  for (auto& ch : chunks) {
    for (size_t i = 0; i < ch.cells.size(); ++i) ql[ch.cells[i]] = (int)i;
    // entry layout: the Zcell column of each (chunk cell, shape) -- its entry relative to the
    // chunk's first, -1 for an entry of a function outside the chunk
    const int64_t f0 = bs->h_fn_ptr[ch.n0], f1 = bs->h_fn_ptr[ch.n1];
    if (entry_layout) {
      zcol_h.assign(ch.cells.size() * nsb, -1);
      for (size_t i = 0; i < ch.cells.size(); ++i)
        for (int j = 0; j < nsb; ++j) {
          const int e = bs->h_cs2e[(int64_t)ch.cells[i] * nsb + j];
          if (e >= f0 && e < f1) zcol_h[i * nsb + j] = (int)(e - f0);
        }
      BEAST_CUDA_TRY(ctx, cudaMemcpyAsync(zcol_d, zcol_h.data(), sizeof(int) * zcol_h.size(), cudaMemcpyHostToDevice, st));
    }
    BEAST_CUDA_TRY(ctx, cudaMemcpyAsync(qcells_d, ch.cells.data(), sizeof(int) * ch.cells.size(), cudaMemcpyHostToDevice, st));
    BEAST_CUDA_TRY(ctx, cudaMemcpyAsync(qlocal_d, ql.data(), sizeof(int) * bs->ncells, cudaMemcpyHostToDevice, st));
    BEAST_CUDA_TRY(ctx, cudaMemsetAsync(counter, 0, sizeof(int), st));
    AsmArgs a;
    a.ss_tabs = &ctx->ss_tabs;
    a.op = to_params(op);
    a.qs = *qs;
    a.ts = ts;
    a.bs = bs;
    a.precision = precision;
    a.qcells = qcells_d;
    a.nq = (int)ch.cells.size();
    a.zcell = zcell;
    a.zcell_fmt = zfmt;
    a.ldc = ldc;
    a.near = nearl;
    a.near_cap = (int)near_cap;
    a.near_count = counter;
    a.flag = ctx->d_flag;
    a.zrow = entry_layout ? ts->zrow_entry : nullptr;
    a.zcol = entry_layout ? zcol_d : nullptr;
    cudaError_t e;
    {
      // algorithmic work: far pairs x flops per pair (EFIE 1200, MFIE 2040, n x K 29600,
      // Helmholtz P0 228 -- per-unit figures from the reference integrands)
      double fpp = op->kind == BEAST_MW_SL ? 1200.0 : op->kind == BEAST_MW_DL ? 2040.0
                 : op->kind == BEAST_MW_NXDL ? 29600.0 : 228.0;
      ProfScope ps(ctx, PK_FAR, fpp * (double)ts->ncells * (double)ch.cells.size());
      e = launch_far(a, ro, ri, st);
    }
    if (e == cudaErrorInvalidValue)
      return beast_fail(ctx, BEAST_ERR_UNSUPPORTED, "operator / space combination not supported");
    BEAST_CUDA_TRY(ctx, e);
    int nnear = 0;
    if (has_near) {
      BEAST_CUDA_TRY(ctx, cudaMemcpyAsync(&nnear, counter, sizeof(int), cudaMemcpyDeviceToHost, st));
      BEAST_CUDA_TRY(ctx, cudaStreamSynchronize(st));
      if (nnear > near_cap) return beast_fail(ctx, BEAST_ERR_ARG, "near-pair list overflow");
      ProfScope ps(ctx, PK_NEAR, (double)nnear, nnear > 0);
      BEAST_CUDA_TRY(ctx, launch_near(a, nnear, ron, rin, ro, ri, st));
    }
    GatherArgs g;
    g.ts = ts;
    g.bs = bs;
    g.zcell = zcell;
    g.zcell_fmt = zfmt;
    g.ldc = ldc;
    g.qlocal = qlocal_d;
    g.tpos = ts->tpos;
    g.n0 = ch.n0;
    g.n1 = ch.n1;
    g.Z = Z;
    g.ldz = ldz;
    g.z_c64 = z_c64;
    g.row_off = row_off;
    g.col_off = col_off;
    g.cr = cr;
    g.ci = ci;
    g.accumulate = accumulate;
    g.entry_layout = entry_layout ? 1 : 0;
    g.f0 = f0;
    {
      // bytes: Zcell chunk read once + output block written (read too when accumulating)
      double by = (double)ldc * nsb * ch.cells.size() * elem +
                  (double)ts->nfuncs * (ch.n1 - ch.n0) * (z_c64 ? 8 : 16) * (accumulate ? 2 : 1);
      ProfScope ps(ctx, PK_GATHER, by);
      BEAST_CUDA_TRY(ctx, launch_gather(g, st));
    }
    for (int c : ch.cells) ql[c] = -1;
  }
  int flag = 0;
  BEAST_CUDA_TRY(ctx, cudaMemcpyAsync(&flag, ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost, st));
  BEAST_CUDA_TRY(ctx, cudaStreamSynchronize(st));
  if (flag & 1) return beast_fail(ctx, BEAST_ERR_ARG, "near-pair list overflow");
  if (flag & 2)
    return beast_fail(ctx, BEAST_ERR_UNSUPPORTED,
                      "singularity extraction not available for this operator/space pairing");
  return BEAST_OK;
}

int beast_assemble(beast_ctx* ctx, const beast_op_desc* op, const beast_qs_desc* qs,
                   const beast_space* ts, const beast_space* bs, int precision, void* Z,
                   int64_t ldz, int z_dtype, int z_loc, int64_t row_off, int64_t col_off,
                   double cr, double ci, int accumulate) {
  ARG_CHECK(ctx, ctx && op && qs && ts && bs && Z, "null argument");
  if (qs->kind == BEAST_QS_TEST_REFINES_TRIAL)
    ARG_CHECK(ctx, bs->mesh->children && ts->kind == BEAST_RT && bs->kind == BEAST_RT,
              "TestRefinesTrialQStrat: RT spaces and the trial mesh's children (beast_mesh_set_children)");
  else if (qs->kind == BEAST_QS_TRIAL_REFINES_TEST)
    ARG_CHECK(ctx, ts->mesh->children && ts->kind == BEAST_RT && bs->kind == BEAST_RT,
              "TrialRefinesTestQStrat: RT spaces and the test mesh's children (beast_mesh_set_children)");
  else
    ARG_CHECK(ctx, ts->mesh == bs->mesh, "test and trial spaces must share the mesh");
  ARG_CHECK(ctx, precision >= BEAST_FP64 && precision <= BEAST_MIXED_BALANCED,
            "unknown precision");
  ARG_CHECK(ctx, z_dtype == BEAST_C128 || z_dtype == BEAST_C64, "unknown matrix dtype");
  ARG_CHECK(ctx, row_off >= 0 && col_off >= 0 && ldz >= row_off + ts->nfuncs, "bad Z addressing");
  ARG_CHECK(ctx, op->kind >= BEAST_MW_SL && op->kind <= BEAST_HH_DLT, "unknown operator kind");
  ARG_CHECK(ctx, qs->kind >= 1 && qs->kind <= 5, "unknown quadrature strategy");
  if (set_device(ctx)) return BEAST_ERR_CUDA;
  const int zc = z_dtype == BEAST_C64;
  if (z_loc == BEAST_DEVICE)
    return assemble_device(ctx, op, qs, ts, bs, precision, Z, ldz, zc, row_off, col_off, cr, ci,
                           accumulate);
  // host Z: assemble the addressed block on the device and copy it out
  const size_t elem = zc ? 8 : 16;
  void* dz = nullptr;
  BEAST_CUDA_TRY(ctx, cudaMallocAsync(&dz, (size_t)ts->nfuncs * bs->nfuncs * elem, ctx->stream));
  char* hz = (char*)Z + (row_off + col_off * ldz) * elem;
  if (accumulate)
    BEAST_CUDA_TRY(ctx, cudaMemcpy2DAsync(dz, ts->nfuncs * elem, hz, ldz * elem, ts->nfuncs * elem,
                                          bs->nfuncs, cudaMemcpyHostToDevice, ctx->stream));
  int rc = assemble_device(ctx, op, qs, ts, bs, precision, dz, ts->nfuncs, zc, 0, 0, cr, ci, accumulate);
  if (rc == BEAST_OK) {
    cudaError_t e = cudaMemcpy2DAsync(hz, ldz * elem, dz, ts->nfuncs * elem, ts->nfuncs * elem,
                                      bs->nfuncs, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) rc = beast_fail(ctx, BEAST_ERR_CUDA, cudaGetErrorString(e));
  }
  cudaFreeAsync(dz, ctx->stream);
  cudaStreamSynchronize(ctx->stream);
  return rc;
}

// ---------------------------------------------------------------------------------------
// block assembly (blockassembler / assemblerow / assemblecol)
// ---------------------------------------------------------------------------------------
// The space restricted to the functions ids[0..nids): the active cells they touch (kept in
// the original active order) and one function per id with its (cell, shape, coefficient)
// entries in the original order, so every entry of the block is computed and summed exactly
// as in the full assembly.  Mirrors reduce_assembly_data (src/bases/basis.jl:486-499), with
// repeated ids kept as separate rows.
static int make_subspace(beast_ctx* ctx, const beast_space* s, const int64_t* ids, int64_t nids,
                         int index_base, beast_space** out) {
  std::vector<int> newc(s->ncells, -1);
  for (int64_t i = 0; i < nids; ++i) {
    const int64_t d = ids[i] - index_base;
    if (d < 0 || d >= s->nfuncs) return beast_fail(ctx, BEAST_ERR_ARG, "block index out of range");
    for (int64_t e = s->h_fn_ptr[d]; e < s->h_fn_ptr[d + 1]; ++e) newc[s->h_fn_cell[e]] = 0;
  }
  std::vector<int> h_cells(s->ncells);
  BEAST_CUDA_TRY(ctx, cudaMemcpy(h_cells.data(), s->cells, sizeof(int) * s->ncells, cudaMemcpyDeviceToHost));
  std::vector<int64_t> mesh_cells;
  for (int64_t c = 0; c < s->ncells; ++c)
    if (newc[c] == 0) {
      newc[c] = (int)mesh_cells.size();
      mesh_cells.push_back(h_cells[c]);
    }
  const int64_t nc = (int64_t)mesh_cells.size();
  if (nc == 0) return beast_fail(ctx, BEAST_ERR_ARG, "block functions have no support");
  const int ns = s->nshapes;
  // (new function, coefficient) per (new cell, shape); each function's entries then come out
  // of the upload's CSR in the full space's (cell, shape) order
  std::vector<std::vector<std::pair<int64_t, double>>> slot(nc * ns);
  for (int64_t i = 0; i < nids; ++i) {
    const int64_t d = ids[i] - index_base;
    for (int64_t e = s->h_fn_ptr[d]; e < s->h_fn_ptr[d + 1]; ++e)
      slot[(int64_t)newc[s->h_fn_cell[e]] * ns + s->h_fn_shape[e]].push_back({i, s->h_fn_coeff[e]});
  }
  int maxfn = 1;
  for (auto& v : slot) maxfn = std::max<int>(maxfn, (int)v.size());
  std::vector<int64_t> ad(nc * ns * maxfn, -1);
  std::vector<double> ac(nc * ns * maxfn, 0.0);
  for (int64_t cs = 0; cs < nc * ns; ++cs)
    for (size_t k = 0; k < slot[cs].size(); ++k) {
      ad[cs * maxfn + k] = slot[cs][k].first;
      ac[cs * maxfn + k] = slot[cs][k].second;
    }
  return beast_space_upload(ctx, s->mesh, s->kind, nc, mesh_cells.data(), maxfn, ns, ad.data(), ac.data(),
                            nids, 0, out);
}

int beast_assemble_block(beast_ctx* ctx, const beast_op_desc* op, const beast_qs_desc* qs,
                         const beast_space* test, const beast_space* trial, const int64_t* test_ids,
                         int64_t ntest, const int64_t* trial_ids, int64_t ntrial, int index_base,
                         int precision, void* Z, int64_t ldz, int z_dtype, int z_loc, double coeff_re,
                         double coeff_im, int accumulate) {
  ARG_CHECK(ctx, ctx && op && qs && test && trial && test_ids && trial_ids && Z, "null argument");
  ARG_CHECK(ctx, ntest > 0 && ntrial > 0 && ldz >= ntest, "invalid block sizes");
  ARG_CHECK(ctx, index_base == 0 || index_base == 1, "index_base must be 0 or 1");
  if (set_device(ctx)) return BEAST_ERR_CUDA;
  beast_space *ts = nullptr, *bs = nullptr;
  int rc = make_subspace(ctx, test, test_ids, ntest, index_base, &ts);
  if (rc == BEAST_OK) rc = make_subspace(ctx, trial, trial_ids, ntrial, index_base, &bs);
  if (rc == BEAST_OK)
    rc = beast_assemble(ctx, op, qs, ts, bs, precision, Z, ldz, z_dtype, z_loc, 0, 0, coeff_re, coeff_im,
                        accumulate);
  beast_space_free(ts);
  beast_space_free(bs);
  return rc;
}

int beast_assemble_local(beast_ctx* ctx, int which, const beast_space* ts, const beast_space* bs,
                         int degree, void* Z, int64_t ldz, int z_dtype, int z_loc, int64_t row_off,
                         int64_t col_off, double cr, double ci) {
  ARG_CHECK(ctx, ctx && ts && bs && Z, "null argument");
  ARG_CHECK(ctx, which == 0 || which == 1, "which must be 0 (Identity) or 1 (NCross)");
  ARG_CHECK(ctx, ts->kind == BEAST_RT && bs->kind == BEAST_RT, "local operators: RT x RT only");
  ARG_CHECK(ctx, ts->mesh == bs->mesh, "test and trial spaces must share the mesh");
  TriRuleDev r;
  ARG_CHECK(ctx, make_trirule(degree, &r), "rule degree not available (1..10)");
  if (set_device(ctx)) return BEAST_ERR_CUDA;
  const int zc = z_dtype == BEAST_C64;
  const size_t elem = zc ? 8 : 16;
  BEAST_CUDA_TRY(ctx, cudaMemsetAsync(ctx->d_flag, 0, sizeof(int), ctx->stream));
  auto flag_check = [&]() -> int {
    int flag = 0;
    BEAST_CUDA_TRY(ctx, cudaMemcpy(&flag, ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost));
    if (flag & 16)
      return beast_fail(ctx, BEAST_ERR_UNSUPPORTED, "local operator: a test function meets more than 64 trial functions");
    return BEAST_OK;
  };
  if (z_loc == BEAST_DEVICE) {
    BEAST_CUDA_TRY(ctx, launch_local_impl(which, ts, bs, bs->cell2act, r, Z, ldz, zc, row_off, col_off,
                                          cr, ci, ctx->d_flag, ctx->stream));
    BEAST_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return flag_check();
  }
  void* dz = nullptr;
  BEAST_CUDA_TRY(ctx, cudaMallocAsync(&dz, (size_t)ts->nfuncs * bs->nfuncs * elem, ctx->stream));
  char* hz = (char*)Z + (row_off + col_off * ldz) * elem;
  BEAST_CUDA_TRY(ctx, cudaMemcpy2DAsync(dz, ts->nfuncs * elem, hz, ldz * elem, ts->nfuncs * elem,
                                        bs->nfuncs, cudaMemcpyHostToDevice, ctx->stream));
  BEAST_CUDA_TRY(ctx, launch_local_impl(which, ts, bs, bs->cell2act, r, dz, ts->nfuncs, zc, 0, 0, cr,
                                        ci, ctx->d_flag, ctx->stream));
  BEAST_CUDA_TRY(ctx, cudaMemcpy2DAsync(hz, ldz * elem, dz, ts->nfuncs * elem, ts->nfuncs * elem,
                                        bs->nfuncs, cudaMemcpyDeviceToHost, ctx->stream));
  BEAST_CUDA_TRY(ctx, cudaFreeAsync(dz, ctx->stream));
  BEAST_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return flag_check();
}

int beast_rhs_planewave(beast_ctx* ctx, int kind, const beast_space* ts, const double* dir,
                        const double* pol, double gr, double gi, double ar, double ai, int degree,
                        double* b, int b_loc) {
  ARG_CHECK(ctx, ctx && ts && dir && b, "null argument");
  ARG_CHECK(ctx, kind >= 0 && kind <= 2, "unknown excitation kind");
  ARG_CHECK(ctx, (kind == BEAST_EXC_HH_DIRICHLET) == (ts->kind != BEAST_RT),
            "excitation kind does not match the test space");
  TriRuleDev r;
  ARG_CHECK(ctx, make_trirule(degree, &r), "rule degree not available (1..10)");
  if (set_device(ctx)) return BEAST_ERR_CUDA;
  double p3[3] = {0, 0, 0};
  if (pol) memcpy(p3, pol, sizeof(p3));
  double* db = b;
  if (b_loc != BEAST_DEVICE) BEAST_CUDA_TRY(ctx, cudaMallocAsync(&db, ts->nfuncs * 16, ctx->stream));
  {
    ProfScope ps(ctx, PK_RHS, (double)ts->nfuncs);
    BEAST_CUDA_TRY(ctx, launch_rhs(kind, ts, dir, p3, gr, gi, ar, ai, r, db, ctx->stream));
  }
  if (b_loc != BEAST_DEVICE) {
    BEAST_CUDA_TRY(ctx, cudaMemcpyAsync(b, db, ts->nfuncs * 16, cudaMemcpyDeviceToHost, ctx->stream));
    BEAST_CUDA_TRY(ctx, cudaFreeAsync(db, ctx->stream));
  }
  BEAST_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return BEAST_OK;
}

int beast_farfield(beast_ctx* ctx, const beast_space* s, const double* u, const double* pts,
                   int64_t npts, double gr, double gi, int degree, double* ff, int loc) {
  ARG_CHECK(ctx, ctx && s && u && pts && ff && npts >= 0, "null argument");
  ARG_CHECK(ctx, s->kind == BEAST_RT, "far field: RT space only");
  TriRuleDev r;
  ARG_CHECK(ctx, make_trirule(degree, &r), "rule degree not available (1..10)");
  if (set_device(ctx)) return BEAST_ERR_CUDA;
  cudaStream_t st = ctx->stream;
  const double *du = u, *dp = pts;
  double* dff = ff;
  void *t1 = nullptr, *t2 = nullptr, *t3 = nullptr;
  if (loc != BEAST_DEVICE) {
    BEAST_CUDA_TRY(ctx, cudaMallocAsync(&t1, s->nfuncs * 16, st));
    BEAST_CUDA_TRY(ctx, cudaMallocAsync(&t2, npts * 24 + 8, st));
    BEAST_CUDA_TRY(ctx, cudaMallocAsync(&t3, npts * 48 + 8, st));
    BEAST_CUDA_TRY(ctx, cudaMemcpyAsync(t1, u, s->nfuncs * 16, cudaMemcpyHostToDevice, st));
    BEAST_CUDA_TRY(ctx, cudaMemcpyAsync(t2, pts, npts * 24, cudaMemcpyHostToDevice, st));
    du = (double*)t1;
    dp = (double*)t2;
    dff = (double*)t3;
  }
  BEAST_CUDA_TRY(ctx, launch_farfield(s, du, dp, npts, gr, gi, r, dff, st));
  if (loc != BEAST_DEVICE) {
    BEAST_CUDA_TRY(ctx, cudaMemcpyAsync(ff, dff, npts * 48, cudaMemcpyDeviceToHost, st));
    cudaFreeAsync(t1, st);
    cudaFreeAsync(t2, st);
    cudaFreeAsync(t3, st);
  }
  BEAST_CUDA_TRY(ctx, cudaStreamSynchronize(st));
  return BEAST_OK;
}

// ---------------------------------------------------------------------------------------
// dense solve
// ---------------------------------------------------------------------------------------
int beast_lu_factor(beast_ctx* ctx, int64_t n, void* A, int64_t lda, int dtype, beast_lu** out) {
  ARG_CHECK(ctx, ctx && A && out && n > 0 && lda >= n, "invalid LU arguments");
  ARG_CHECK(ctx, dtype == BEAST_C128 || dtype == BEAST_C64, "unknown dtype");
  if (set_device(ctx)) return BEAST_ERR_CUDA;
  beast_lu* lu = new beast_lu();
  lu->ctx = ctx;
  lu->n = n;
  lu->lda = lda;
  lu->dtype = dtype;
  lu->A = A;
  cudaError_t e = cudaMalloc(&lu->ipiv, lu_aux_bytes(n, dtype));
  if (e != cudaSuccess) {
    delete lu;
    return beast_fail(ctx, BEAST_ERR_OOM, "pivot allocation failed");
  }
  int rc = lu_factor_dev(ctx, n, A, lda, dtype, lu->ipiv, &lu->info);
  if (rc) {
    beast_lu_free(lu);
    return rc;
  }
  *out = lu;
  if (lu->info > 0)
    return beast_fail(ctx, BEAST_ERR_SINGULAR, "exactly singular pivot in column " + std::to_string(lu->info));
  return BEAST_OK;
}

int beast_lu_solve(beast_ctx* ctx, const beast_lu* lu, int64_t nrhs, void* B, int64_t ldb) {
  ARG_CHECK(ctx, ctx && lu && B && nrhs >= 0 && ldb >= lu->n, "invalid solve arguments");
  if (set_device(ctx)) return BEAST_ERR_CUDA;
  int rc = lu_solve_dev(ctx, lu->n, lu->A, lu->lda, lu->dtype, lu->ipiv, B, ldb, nrhs);
  if (rc) return rc;
  return trsv_check(ctx);
}

int beast_lu_free(beast_lu* lu) {
  if (!lu) return BEAST_OK;
  cudaSetDevice(lu->ctx->device);
  cudaStreamSynchronize(lu->ctx->stream);
  if (lu->ipiv) cudaFree(lu->ipiv);
  delete lu;
  return BEAST_OK;
}

static double dev_norm(beast_ctx* ctx, int64_t n, const double* x, double* scratch) {
  vec_norm2(n, x, scratch, ctx->stream);
  double h = 0;
  cudaMemcpyAsync(&h, scratch, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
  cudaStreamSynchronize(ctx->stream);
  return std::sqrt(h);
}

// copy A into F (c64 for the mixed path, c128 otherwise) and factor F in place
static int factor_copy(beast_ctx* ctx, int64_t n, const void* A, int64_t lda, int a_dtype, void* F,
                       int fdt, bool pivot, bool sym, beast_lu** out) {
  cudaStream_t st = ctx->stream;
  if (fdt == BEAST_C64) {
    if (a_dtype == BEAST_C64 && sym) {  // the symmetric factorisation reads the block-lower part only
      ProfScope ps(ctx, PK_CONVERT, (double)n * n * 8);
      BEAST_CUDA_TRY(ctx, copy_lower_c64(n, A, lda, F, n, st));
    } else if (a_dtype == BEAST_C64) {
      BEAST_CUDA_TRY(ctx, cudaMemcpy2DAsync(F, n * 8, A, lda * 8, n * 8, n, cudaMemcpyDeviceToDevice, st));
    } else if (sym) {
      ProfScope ps(ctx, PK_CONVERT, (double)n * n * 12);
      BEAST_CUDA_TRY(ctx, convert_lower_c128_to_c64(n, A, lda, F, n, st));
    } else {
      ProfScope ps(ctx, PK_CONVERT, (double)n * n * 24);
      BEAST_CUDA_TRY(ctx, convert_c128_to_c64(n, n, (const double*)A, lda, (float*)F, n, st));
    }
  } else {
    ARG_CHECK(ctx, a_dtype == BEAST_C128, "plain FP64 solve needs a c128 matrix");
    BEAST_CUDA_TRY(ctx, cudaMemcpy2DAsync(F, n * 16, A, lda * 16, n * 16, n, cudaMemcpyDeviceToDevice, st));
  }
  beast_lu* lu = new beast_lu();
  lu->ctx = ctx;
  lu->n = n;
  lu->lda = n;
  lu->dtype = fdt;
  lu->A = F;
  cudaError_t e = cudaMalloc(&lu->ipiv, lu_aux_bytes(n, fdt));
  if (e != cudaSuccess) {
    delete lu;
    return beast_fail(ctx, BEAST_ERR_OOM, "pivot allocation failed");
  }
  int rc = lu_factor_dev(ctx, n, F, n, fdt, lu->ipiv, &lu->info, pivot, sym);
  if (rc == BEAST_OK && lu->info > 0)
    rc = beast_fail(ctx, BEAST_ERR_SINGULAR, "zero pivot in column " + std::to_string(lu->info));
  if (rc) {
    beast_lu_free(lu);
    return rc;
  }
  *out = lu;
  return BEAST_OK;
}

// ---- factored systems: the matrix A (as stored) and the factors of its copy F
// FP64: partial-pivoting LU in complex FP64 (zgetrf semantics) of a c128 copy.
// MIXED: complex FP32 factorisation (tensor-core trailing updates) of a c64 copy, FP64
// iterative refinement against A as stored.  Factorisations tried in turn, each taking over
// when the previous one meets a zero pivot or its refinement diverges or stagnates:
//   symmetric (LDL^T-type, half the work; only when A is complex symmetric to within 1e-2
//   in a sampled Frobenius measure -- e.g. a Galerkin EFIE matrix, symmetric up to quadrature),
//   unpivoted LU, LU with partial pivoting.
struct DenseSystem {
  int64_t n = 0, lda = 0;
  const void* A = nullptr;
  int a_dtype = 0;
  bool mixed = false;
  void* F = nullptr;        // factor copy (stream-ordered pool memory)
  beast_lu* lu = nullptr;
  int mode = 0;             // 2 symmetric, 1 unpivoted LU, 0 LU with partial pivoting
};

static void system_release(beast_ctx* ctx, DenseSystem& S) {
  if (S.lu) beast_lu_free(S.lu);
  S.lu = nullptr;
  if (S.F) cudaFreeAsync(S.F, ctx->stream);
  S.F = nullptr;
}

// the factor copy of A in mode S.mode (allocated on first use)
static int system_factor(beast_ctx* ctx, DenseSystem& S) {
  cudaStream_t st = ctx->stream;
  const int64_t n = S.n;
  const size_t fel = S.mixed ? 8 : 16;
  if (S.lu) {
    beast_lu_free(S.lu);
    S.lu = nullptr;
  }
  if (!S.F) {
    // the assembly workspace (kept by the context) and the device pool's freed blocks stay
    // mapped; when the factor copy would not fit next to them, hand them back first (the
    // next assembly grows its workspace again)
    size_t fr = 0, tot = 0;
    const size_t want = (size_t)n * n * fel + ((size_t)1 << 31);
    if (cudaMemGetInfo(&fr, &tot) == cudaSuccess && fr < want) {
      cudaMemPool_t pool;
      BEAST_CUDA_TRY(ctx, cudaStreamSynchronize(st));
      if (ctx->ws) {
        cudaFree(ctx->ws);
        ctx->ws = nullptr;
        ctx->ws_size = 0;
      }
      if (cudaDeviceGetDefaultMemPool(&pool, ctx->device) == cudaSuccess) cudaMemPoolTrimTo(pool, 0);
    }
    BEAST_CUDA_TRY(ctx, cudaMallocAsync(&S.F, (size_t)n * n * fel, st));
  }
  ctx->last_factor_mode = S.mode;
  return factor_copy(ctx, n, S.A, S.lda, S.a_dtype, S.F, S.mixed ? BEAST_C64 : BEAST_C128, S.mode == 0, S.mode == 2,
                     &S.lu);
}

// factor A: the first mode of the sequence that factors without a zero pivot
static int system_setup(beast_ctx* ctx, DenseSystem& S, int64_t n, const void* A, int64_t lda, int a_dtype,
                        bool mixed) {
  S.n = n;
  S.lda = lda;
  S.A = A;
  S.a_dtype = a_dtype;
  S.mixed = mixed;
  S.mode = mixed ? (asym_sample(ctx, n, A, lda, a_dtype) <= 1e-2 ? 2 : 1) : 0;
  for (;;) {
    int rc = system_factor(ctx, S);
    if (rc == BEAST_ERR_SINGULAR && S.mode > 0) {
      --S.mode;
      continue;
    }
    return rc;
  }
}

// x = A \ b for device vectors (b, x: c128 [n x nrhs], ld n) with the factors of S; on the
// mixed path a refinement that stagnates or diverges moves S to the next factorisation mode
// and starts over, so the result never depends on a cheaper factorisation being good
static int system_solve(beast_ctx* ctx, DenseSystem& S, const double* b, double* x, int64_t nrhs, double tol,
                        int maxiter, int* iters, double* resid) {
  cudaStream_t st = ctx->stream;
  const int64_t n = S.n;
  double *r = nullptr, *d = nullptr, *nrm = nullptr;
  float* d32 = nullptr;
  BEAST_CUDA_TRY(ctx, cudaMallocAsync(&r, n * 16, st));
  BEAST_CUDA_TRY(ctx, cudaMallocAsync(&d, n * 16, st));
  BEAST_CUDA_TRY(ctx, cudaMallocAsync(&nrm, 64, st));
  if (S.mixed) BEAST_CUDA_TRY(ctx, cudaMallocAsync(&d32, n * 8, st));
  int it_max = 0;
  double res_max = 0;
  int rc = BEAST_OK;
  ctx->last_factor_mode = S.mode;
  for (;;) {
    it_max = 0;
    res_max = 0;
    bool retry = false;
    for (int64_t k = 0; k < nrhs && rc == BEAST_OK; ++k) {
      const double* bk = b + 2 * k * n;
      double* xk = x + 2 * k * n;
      double bn = dev_norm(ctx, n, bk, nrm);
      if (!S.mixed) {
        BEAST_CUDA_TRY(ctx, vec_copy(n, bk, xk, st));
        rc = lu_solve_dev(ctx, n, S.F, n, BEAST_C128, S.lu->ipiv, xk, n, 1);
        if (rc) break;
        BEAST_CUDA_TRY(ctx, vec_copy(n, bk, r, st));
        {
          ProfScope ps(ctx, PK_GEMV, (double)n * n * 16, 2);
          BEAST_CUDA_TRY(ctx, gemv_dev(n, S.A, S.lda, 0, xk, r, -1.0, 1.0, st));
        }
        double rn = dev_norm(ctx, n, r, nrm);
        if ((rc = trsv_check(ctx))) break;
        res_max = std::max(res_max, bn > 0 ? rn / bn : rn);
        continue;
      }
      BEAST_CUDA_TRY(ctx, cudaMemsetAsync(xk, 0, n * 16, st));
      BEAST_CUDA_TRY(ctx, vec_copy(n, bk, r, st));
      int it = 0;
      double rel = 1.0, prev = 1e300;
      int slow = 0;
      while (true) {
        BEAST_CUDA_TRY(ctx, convert_c128_to_c64(n, 1, r, n, d32, n, st));
        rc = lu_solve_dev(ctx, n, S.F, n, BEAST_C64, S.lu->ipiv, d32, n, 1);
        if (rc) break;
        BEAST_CUDA_TRY(ctx, convert_c64_to_c128(n, 1, d32, n, d, n, st));
        BEAST_CUDA_TRY(ctx, vec_axpy(n, 1.0, 0.0, d, xk, st));
        BEAST_CUDA_TRY(ctx, vec_copy(n, bk, r, st));
        {
          ProfScope ps(ctx, PK_GEMV, (double)n * n * (S.a_dtype == BEAST_C64 ? 8 : 16), 2);
          BEAST_CUDA_TRY(ctx, gemv_dev(n, S.A, S.lda, S.a_dtype == BEAST_C64, xk, r, -1.0, 1.0, st));
        }
        ++it;
        double rn = dev_norm(ctx, n, r, nrm);
        if ((rc = trsv_check(ctx))) break;
        rel = bn > 0 ? rn / bn : rn;
        if (rel <= tol || it >= maxiter) break;
        // contraction slower than 1/2 per step twice in a row: the factors are not good enough
        if (!(rel < 0.5 * prev)) ++slow; else slow = 0;
        if (!std::isfinite(rel) || slow >= 2) break;
        prev = rel;
      }
      if (rc) break;
      it_max = std::max(it_max, it);
      res_max = std::isfinite(rel) ? std::max(res_max, rel) : rel;
      if (!(rel <= tol)) {  // also a non-finite residual
        if (S.mode > 0) retry = true;
        else rc = beast_fail(ctx, BEAST_ERR_NOCONV, "iterative refinement did not reach the tolerance");
      }
    }
    if (retry && rc == BEAST_OK) {
      // the next factorisation mode; a zero pivot there moves on again
      for (;;) {
        --S.mode;
        rc = system_factor(ctx, S);
        if (rc == BEAST_ERR_SINGULAR && S.mode > 0) {
          rc = BEAST_OK;
          continue;
        }
        break;
      }
      if (rc) break;
      continue;
    }
    break;
  }
  cudaFreeAsync(r, st);
  cudaFreeAsync(d, st);
  cudaFreeAsync(nrm, st);
  if (d32) cudaFreeAsync(d32, st);
  if (iters) *iters = it_max;
  if (resid) *resid = res_max;
  return rc;
}

// core of the dense solve on device vectors (b, x: c128 [n x nrhs], ld n)
static int solve_dense_device(beast_ctx* ctx, int64_t n, const void* A, int64_t lda, int a_dtype,
                              int precision, const double* b, double* x, int64_t nrhs, double tol,
                              int maxiter, int* iters, double* resid) {
  DenseSystem S;
  int rc = system_setup(ctx, S, n, A, lda, a_dtype, precision == BEAST_MIXED);
  if (rc == BEAST_OK) rc = system_solve(ctx, S, b, x, nrhs, tol, maxiter, iters, resid);
  system_release(ctx, S);
  cudaStreamSynchronize(ctx->stream);
  return rc;
}

int beast_solve_dense(beast_ctx* ctx, int64_t n, const void* A, int64_t lda, int a_dtype,
                      int precision, const double* b, double* x, int64_t nrhs, int bx_loc,
                      double tol, int maxiter, int* iters, double* resid) {
  ARG_CHECK(ctx, ctx && A && b && x && n > 0 && lda >= n && nrhs >= 1, "invalid solve arguments");
  ARG_CHECK(ctx, precision >= BEAST_FP64 && precision <= BEAST_MIXED_BALANCED,
            "unknown precision");
  if (precision == BEAST_MIXED_ACCURATE || precision == BEAST_MIXED_BALANCED) precision = BEAST_MIXED;  // mixed factorisation
  if (set_device(ctx)) return BEAST_ERR_CUDA;
  if (maxiter <= 0) maxiter = 30;
  if (tol <= 0) tol = 1e-12;
  if (bx_loc == BEAST_DEVICE)
    return solve_dense_device(ctx, n, A, lda, a_dtype, precision, b, x, nrhs, tol, maxiter, iters, resid);
  double *db = nullptr, *dx = nullptr;
  cudaStream_t st = ctx->stream;
  BEAST_CUDA_TRY(ctx, cudaMallocAsync(&db, n * nrhs * 16, st));
  BEAST_CUDA_TRY(ctx, cudaMallocAsync(&dx, n * nrhs * 16, st));
  BEAST_CUDA_TRY(ctx, cudaMemcpyAsync(db, b, n * nrhs * 16, cudaMemcpyHostToDevice, st));
  int rc = solve_dense_device(ctx, n, A, lda, a_dtype, precision, db, dx, nrhs, tol, maxiter, iters, resid);
  if (rc == BEAST_OK || rc == BEAST_ERR_NOCONV)
    cudaMemcpyAsync(x, dx, n * nrhs * 16, cudaMemcpyDeviceToHost, st);
  cudaFreeAsync(db, st);
  cudaFreeAsync(dx, st);
  cudaStreamSynchronize(st);
  return rc;
}

// restarted GMRES with modified Gram-Schmidt (one dot kernel per basis vector) and Givens
// rotations on the host (the Hessenberg matrix is tiny)
int beast_gmres(beast_ctx* ctx, int64_t n, const void* A, int64_t lda, int a_dtype, const double* b,
                double* x, int bx_loc, double reltol, int restart, int maxiter, int* iters,
                double* resid) {
  ARG_CHECK(ctx, ctx && A && b && x && n > 0 && lda >= n, "invalid GMRES arguments");
  if (set_device(ctx)) return BEAST_ERR_CUDA;
  cudaStream_t st = ctx->stream;
  if (restart <= 0) restart = (int)std::min<int64_t>(n, 200);
  if (maxiter <= 0) maxiter = (int)n;
  const int m = restart;
  double *V = nullptr, *w = nullptr, *db = nullptr, *dx = nullptr, *h = nullptr, *nrm = nullptr;
  BEAST_CUDA_TRY(ctx, cudaMallocAsync(&V, (size_t)n * (m + 1) * 16, st));
  BEAST_CUDA_TRY(ctx, cudaMallocAsync(&w, n * 16, st));
  BEAST_CUDA_TRY(ctx, cudaMallocAsync(&h, (m + 2) * 16, st));
  BEAST_CUDA_TRY(ctx, cudaMallocAsync(&nrm, 64, st));
  if (bx_loc != BEAST_DEVICE) {
    BEAST_CUDA_TRY(ctx, cudaMallocAsync(&db, n * 16, st));
    BEAST_CUDA_TRY(ctx, cudaMallocAsync(&dx, n * 16, st));
    BEAST_CUDA_TRY(ctx, cudaMemcpyAsync(db, b, n * 16, cudaMemcpyHostToDevice, st));
  } else {
    db = (double*)b;
    dx = x;
  }
  BEAST_CUDA_TRY(ctx, cudaMemsetAsync(dx, 0, n * 16, st));
  typedef std::complex<double> cd;
  double bn = dev_norm(ctx, n, db, nrm);
  int it = 0;
  double rel = 1.0;
  std::vector<cd> H((size_t)(m + 1) * m), cs(m), sn(m), g(m + 1), y(m), hh(m + 1);
  while (true) {
    // r = b - A x  into V[:,0]
    BEAST_CUDA_TRY(ctx, vec_copy(n, db, V, st));
    BEAST_CUDA_TRY(ctx, gemv_dev(n, A, lda, a_dtype == BEAST_C64, dx, V, -1.0, 1.0, st));
    double rn = dev_norm(ctx, n, V, nrm);
    rel = bn > 0 ? rn / bn : rn;
    if (rel <= reltol || it >= maxiter || rn == 0.0) break;
    BEAST_CUDA_TRY(ctx, vec_axpy(n, 1.0 / rn - 1.0, 0.0, V, V, st));  // V0 *= 1/rn
    std::fill(g.begin(), g.end(), cd(0));
    g[0] = rn;
    int k = 0;
    for (; k < m && it < maxiter; ++k) {
      double* vk = V + 2 * (int64_t)k * n;
      double* vk1 = V + 2 * (int64_t)(k + 1) * n;
      BEAST_CUDA_TRY(ctx, gemv_dev(n, A, lda, a_dtype == BEAST_C64, vk, w, 1.0, 0.0, st));
      // modified Gram-Schmidt as two classical passes (reorthogonalisation), FP64
      for (int pass = 0; pass < 2; ++pass) {
        BEAST_CUDA_TRY(ctx, vec_dots(n, k + 1, V, n, w, h, st));
        BEAST_CUDA_TRY(ctx, vec_gemv_sub(n, k + 1, V, n, h, w, st));
        BEAST_CUDA_TRY(ctx, cudaMemcpyAsync(hh.data(), h, (k + 1) * 16, cudaMemcpyDeviceToHost, st));
        BEAST_CUDA_TRY(ctx, cudaStreamSynchronize(st));
        for (int j = 0; j <= k; ++j) {
          if (pass == 0)
            H[j + (size_t)k * (m + 1)] = hh[j];
          else
            H[j + (size_t)k * (m + 1)] += hh[j];
        }
      }
      double hn = dev_norm(ctx, n, w, nrm);
      H[k + 1 + (size_t)k * (m + 1)] = hn;
      BEAST_CUDA_TRY(ctx, cudaMemsetAsync(vk1, 0, n * 16, st));
      if (hn > 0) BEAST_CUDA_TRY(ctx, vec_axpy(n, 1.0 / hn, 0.0, w, vk1, st));
      for (int j = 0; j < k; ++j) {
        cd h0 = H[j + (size_t)k * (m + 1)], h1 = H[j + 1 + (size_t)k * (m + 1)];
        H[j + (size_t)k * (m + 1)] = std::conj(cs[j]) * h0 + std::conj(sn[j]) * h1;
        H[j + 1 + (size_t)k * (m + 1)] = -sn[j] * h0 + cs[j] * h1;
      }
      cd h0 = H[k + (size_t)k * (m + 1)], h1 = H[k + 1 + (size_t)k * (m + 1)];
      double den = std::sqrt(std::norm(h0) + std::norm(h1));
      cs[k] = den > 0 ? h0 / den : cd(1);
      sn[k] = den > 0 ? h1 / den : cd(0);
      H[k + (size_t)k * (m + 1)] = den;
      g[k + 1] = -sn[k] * g[k];
      g[k] = std::conj(cs[k]) * g[k];
      ++it;
      if (std::abs(g[k + 1]) <= reltol * bn) {
        ++k;
        break;
      }
    }
    for (int j = k - 1; j >= 0; --j) {
      cd s = g[j];
      for (int l = j + 1; l < k; ++l) s -= H[j + (size_t)l * (m + 1)] * y[l];
      y[j] = s / H[j + (size_t)j * (m + 1)];
    }
    std::vector<double> yh(2 * k);
    for (int j = 0; j < k; ++j) {
      yh[2 * j] = -y[j].real();  // vec_gemv_sub subtracts
      yh[2 * j + 1] = -y[j].imag();
    }
    BEAST_CUDA_TRY(ctx, cudaMemcpyAsync(h, yh.data(), k * 16, cudaMemcpyHostToDevice, st));
    BEAST_CUDA_TRY(ctx, vec_gemv_sub(n, k, V, n, h, dx, st));
  }
  if (bx_loc != BEAST_DEVICE) BEAST_CUDA_TRY(ctx, cudaMemcpyAsync(x, dx, n * 16, cudaMemcpyDeviceToHost, st));
  BEAST_CUDA_TRY(ctx, cudaStreamSynchronize(st));
  cudaFreeAsync(V, st);
  cudaFreeAsync(w, st);
  cudaFreeAsync(h, st);
  cudaFreeAsync(nrm, st);
  if (bx_loc != BEAST_DEVICE) {
    cudaFreeAsync(db, st);
    cudaFreeAsync(dx, st);
  }
  cudaStreamSynchronize(st);
  if (iters) *iters = it;
  if (resid) *resid = rel;
  if (rel > reltol) return beast_fail(ctx, BEAST_ERR_NOCONV, "GMRES did not converge");
  return BEAST_OK;
}

}  // extern "C"

// a batch of P0 jobs assembled by one persistent launch (beast_batch_*)
struct beast_batch {
  beast_ctx* ctx = nullptr;
  BatchLaunch L;
  BatchJobDev* jobs = nullptr;
  BatchTile* tiles = nullptr;
  NearPairB* near = nullptr;
  int* counter = nullptr;  // [0] near-pair count, [1] status
  std::vector<void*> zcols;  // the jobs' column maps
  cudaGraphExec_t exec = nullptr;
};

// an assembled and factored system kept on the device (beast_system_*)
struct beast_system {
  beast_ctx* ctx = nullptr;
  const beast_space* space = nullptr;
  int precision = 0;
  int dtype = 0;
  void* Z = nullptr;
  DenseSystem S;
  size_t bytes = 0;
};

extern "C" {

int beast_system_create(beast_ctx* ctx, const beast_op_desc* op, const beast_qs_desc* qs, const beast_space* space,
                        int local_which, double local_re, double local_im, int precision, beast_system** out) {
  ARG_CHECK(ctx, ctx && op && qs && space && out, "null argument");
  ARG_CHECK(ctx, precision >= BEAST_FP64 && precision <= BEAST_MIXED_BALANCED,
            "unknown precision");
  ARG_CHECK(ctx, local_which >= -1 && local_which <= 1, "local_which must be -1 (none), 0 (Identity) or 1 (NCross)");
  if (set_device(ctx)) return BEAST_ERR_CUDA;
  cudaStream_t st = ctx->stream;
  const int64_t n = space->nfuncs;
  beast_system* y = new beast_system();
  y->ctx = ctx;
  y->space = space;
  y->precision = precision;
  y->dtype = precision == BEAST_MIXED ? BEAST_C64 : BEAST_C128;
  const size_t el = y->dtype == BEAST_C64 ? 8 : 16;
  cudaError_t e = cudaMallocAsync(&y->Z, (size_t)n * n * el, st);
  if (e != cudaSuccess) {
    delete y;
    return beast_fail(ctx, BEAST_ERR_OOM, "system matrix allocation failed");
  }
  int rc = beast_assemble(ctx, op, qs, space, space, precision, y->Z, n, y->dtype, BEAST_DEVICE, 0, 0, 1.0, 0.0, 0);
  if (rc == BEAST_OK && local_which >= 0)
    rc = beast_assemble_local(ctx, local_which, space, space, 6, y->Z, n, y->dtype, BEAST_DEVICE, 0, 0, local_re,
                              local_im);
  if (rc == BEAST_OK) rc = system_setup(ctx, y->S, n, y->Z, n, y->dtype, precision != BEAST_FP64);
  if (rc == BEAST_OK) rc = beast_ctx_synchronize(ctx);
  if (rc) {
    beast_system_free(y);
    return rc;
  }
  y->bytes = (size_t)n * n * el + (size_t)n * n * (precision == BEAST_FP64 ? 16 : 8) + lu_aux_bytes(n, y->S.mixed ? BEAST_C64 : BEAST_C128);
  *out = y;
  return BEAST_OK;
}

int beast_system_solve(beast_ctx* ctx, beast_system* y, int exc_kind, int64_t nrhs, const double* dirs,
                       const double* pols, double egr, double egi, double tol, double* x, int x_loc, int* iters,
                       double* resid) {
  ARG_CHECK(ctx, ctx && y && dirs && x && nrhs >= 1, "invalid system solve arguments");
  ARG_CHECK(ctx, y->ctx == ctx, "the system belongs to another context");
  if (set_device(ctx)) return BEAST_ERR_CUDA;
  cudaStream_t st = ctx->stream;
  const int64_t n = y->S.n;
  double *b = nullptr, *dx = nullptr;
  BEAST_CUDA_TRY(ctx, cudaMallocAsync(&b, n * nrhs * 16, st));
  BEAST_CUDA_TRY(ctx, cudaMallocAsync(&dx, n * nrhs * 16, st));
  int rc = BEAST_OK;
  TriRuleDev r;
  make_trirule(8, &r);
  for (int64_t k = 0; k < nrhs && rc == BEAST_OK; ++k) {
    double p3[3] = {0, 0, 0};
    if (pols) memcpy(p3, pols + 3 * k, sizeof(p3));
    ProfScope ps(ctx, PK_RHS, (double)n);
    cudaError_t e = launch_rhs(exc_kind, y->space, dirs + 3 * k, p3, egr, egi, 1.0, 0.0, r, b + 2 * k * n, st);
    if (e != cudaSuccess) rc = beast_fail(ctx, BEAST_ERR_CUDA, cudaGetErrorString(e));
  }
  if (rc == BEAST_OK) rc = system_solve(ctx, y->S, b, dx, nrhs, tol > 0 ? tol : 1e-12, 30, iters, resid);
  if (rc == BEAST_OK || rc == BEAST_ERR_NOCONV)
    cudaMemcpyAsync(x, dx, n * nrhs * 16, x_loc == BEAST_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                    st);
  cudaFreeAsync(b, st);
  cudaFreeAsync(dx, st);
  cudaStreamSynchronize(st);
  return rc;
}

int beast_system_bytes(const beast_system* y, size_t* bytes) {
  if (!y || !bytes) return BEAST_ERR_ARG;
  *bytes = y->bytes;
  return BEAST_OK;
}

int beast_system_free(beast_system* y) {
  if (!y) return BEAST_OK;
  beast_ctx* ctx = y->ctx;
  cudaSetDevice(ctx->device);
  system_release(ctx, y->S);
  if (y->Z) cudaFreeAsync(y->Z, ctx->stream);
  cudaStreamSynchronize(ctx->stream);
  delete y;
  return BEAST_OK;
}

int beast_batch_create(beast_ctx* ctx, const beast_qs_desc* qs, int64_t njobs, const beast_space* const* spaces,
                       const beast_op_desc* ops, void* const* Z, int precision, int tile_m, int tile_q, int order,
                       beast_batch** out) {
  ARG_CHECK(ctx, ctx && qs && spaces && ops && Z && out && njobs > 0, "null argument");
  ARG_CHECK(ctx, precision >= BEAST_FP64 && precision <= BEAST_MIXED_BALANCED,
            "unknown precision");
  ARG_CHECK(ctx, order >= 0 && order <= 2, "order must be 0, 1 or 2");
  if (tile_m <= 0) tile_m = 128;
  if (tile_q <= 0) tile_q = 16;
  ARG_CHECK(ctx, tile_m <= 1024 && tile_q <= 256, "tile shape out of range");
  const int kind = ops[0].kind;
  ARG_CHECK(ctx, kind == BEAST_HH_SL || kind == BEAST_HH_DLT,
            "batched assembly: Helmholtz single layer or transposed double layer");
  for (int64_t j = 0; j < njobs; ++j) {
    const beast_space* s = spaces[j];
    ARG_CHECK(ctx, s && Z[j] && ops[j].kind == kind, "every job needs a space, a matrix and the batch's operator");
    ARG_CHECK(ctx, s->kind == BEAST_P0 && s->injective && s->maxfn == 1 &&
                       (int64_t)s->h_fn_cell.size() == s->ncells && s->nfuncs == s->ncells,
              "batched assembly: P0 spaces with one function per cell");
    for (double c : s->h_fn_coeff) ARG_CHECK(ctx, c == 1.0, "batched assembly: P0 coefficients must be 1");
  }
  TriRuleDev ro, ri, ron, rin;
  ARG_CHECK(ctx, make_trirule(qs->outer_far, &ro) && make_trirule(qs->inner_far, &ri), "far rule degree not available");
  if (qs->kind == BEAST_QS_WILTON_SAUTER) {
    ARG_CHECK(ctx, make_trirule(qs->outer_near, &ron) && make_trirule(qs->inner_near, &rin), "near rule degree not available");
  } else {
    ron = ro;
    rin = ri;
  }
  if (set_device(ctx)) return BEAST_ERR_CUDA;
  beast_batch* b = new beast_batch();
  b->ctx = ctx;
  // job table and zcol (= the cell's entry: with one cell per function, its function)
  std::vector<BatchJobDev> jt(njobs);
  std::vector<std::vector<int>> cols(njobs);
  int64_t near_cap = 0;
  cudaError_t e = cudaSuccess;
  for (int64_t j = 0; j < njobs && e == cudaSuccess; ++j) {
    const beast_space* s = spaces[j];
    int* zc = nullptr;
    e = cudaMalloc(&zc, sizeof(int) * s->ncells);
    if (e == cudaSuccess) {
      b->zcols.push_back(zc);
      e = cudaMemcpy(zc, s->h_cs2e.data(), sizeof(int) * s->ncells, cudaMemcpyHostToDevice);
    }
    BatchJobDev& J = jt[j];
    J.op = to_params(&ops[j]);
    J.k2 = ops[j].gamma_re * ops[j].gamma_re + ops[j].gamma_im * ops[j].gamma_im;
    J.geo = s->geo;
    J.geof = s->geof;
    J.tperm = s->tperm;
    J.zrow = s->zrow_entry;
    J.zcol = zc;
    J.ncells = s->ncells;
    J.Z = Z[j];
    J.ldz = s->nfuncs;
    near_cap += 48 * s->ncells;
  }
  // tile list in the requested order
  std::vector<int64_t> jord(njobs);
  for (int64_t j = 0; j < njobs; ++j) jord[j] = j;
  if (order == 1)
    std::stable_sort(jord.begin(), jord.end(), [&](int64_t a, int64_t c) { return jt[a].ncells > jt[c].ncells; });
  std::vector<BatchTile> tiles;
  if (order == 2) {
    std::vector<std::vector<BatchTile>> per(njobs);
    size_t most = 0;
    for (int64_t j = 0; j < njobs; ++j) {
      for (int64_t p0 = 0; p0 < jt[j].ncells; p0 += tile_m)
        for (int64_t q0 = 0; q0 < jt[j].ncells; q0 += tile_q) per[j].push_back(BatchTile{(int)j, (int)p0, (int)q0, 0});
      most = std::max(most, per[j].size());
    }
    for (size_t k = 0; k < most; ++k)
      for (int64_t j = 0; j < njobs; ++j)
        if (k < per[j].size()) tiles.push_back(per[j][k]);
  } else {
    for (int64_t j : jord)
      for (int64_t p0 = 0; p0 < jt[j].ncells; p0 += tile_m)
        for (int64_t q0 = 0; q0 < jt[j].ncells; q0 += tile_q) tiles.push_back(BatchTile{(int)j, (int)p0, (int)q0, 0});
  }
  if (e == cudaSuccess) e = cudaMalloc(&b->jobs, sizeof(BatchJobDev) * njobs);
  if (e == cudaSuccess) e = cudaMemcpy(b->jobs, jt.data(), sizeof(BatchJobDev) * njobs, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMalloc(&b->tiles, sizeof(BatchTile) * std::max<size_t>(1, tiles.size()));
  if (e == cudaSuccess && !tiles.empty())
    e = cudaMemcpy(b->tiles, tiles.data(), sizeof(BatchTile) * tiles.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMalloc(&b->near, sizeof(NearPairB) * near_cap);
  if (e == cudaSuccess) e = cudaMalloc(&b->counter, 256);
  b->L.jobs = b->jobs;
  if (e != cudaSuccess) {
    beast_batch_free(b);
    return beast_fail(ctx, e == cudaErrorMemoryAllocation ? BEAST_ERR_OOM : BEAST_ERR_CUDA,
                      std::string("batch setup: ") + cudaGetErrorString(e));
  }
  BatchLaunch& L = b->L;
  L.tiles = b->tiles;
  L.ntiles = (int)tiles.size();
  L.qs_kind = qs->kind;
  L.qs = *qs;
  L.ro = ro;
  L.ri = ri;
  L.ron = ron;
  L.rin = rin;
  L.precision = precision;
  L.zfmt = precision == BEAST_MIXED ? ZCELL_C64 : ZCELL_C128;
  L.op_kind = kind;
  L.near = b->near;
  L.near_cap = (int)std::min<int64_t>(near_cap, INT32_MAX);
  L.near_count = b->counter;
  L.flag = b->counter + 1;
  L.tile_m = tile_m;
  L.tile_q = tile_q;
  // persistent grids: a few CTAs per SM (the far kernel holds ~130 registers per thread)
  L.grid_far = std::max(1, std::min(L.ntiles, ctx->num_sms * std::max(1, 512 / std::max(64, tile_m))));
  L.grid_near = ctx->num_sms * 8;
  // the single layer's Sauter-Schwab pairs in double-float off the FP64 path: node tables now
  // (graph capture comes later)
  if (kind == BEAST_HH_SL && precision != BEAST_FP64 && qs->kind != BEAST_QS_DOUBLENUM) {
    cudaError_t e = ss_tables(&ctx->ss_tabs, *qs, ctx->stream, L.ssdf_tab, L.ssdf_items);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
      beast_batch_free(b);
      return beast_fail(ctx, BEAST_ERR_CUDA, std::string("batch node tables: ") + cudaGetErrorString(e));
    }
    L.ssdf = 1;
  }
  *out = b;
  return BEAST_OK;
}

int beast_batch_assemble(beast_ctx* ctx, beast_batch* b) {
  ARG_CHECK(ctx, ctx && b && b->ctx == ctx, "invalid batch");
  if (set_device(ctx)) return BEAST_ERR_CUDA;
  cudaStream_t st = ctx->stream;
  if (!b->exec) {
    BEAST_CUDA_TRY(ctx, upload_tables(st));
    BEAST_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    // capture on a stream of our own (a capture cannot run on the legacy default stream)
    cudaStream_t cs;
    BEAST_CUDA_TRY(ctx, cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->counter, 0, 2 * sizeof(int), cs);
    if (e == cudaSuccess) e = launch_far_batch(b->L, cs);
    if (e == cudaSuccess) e = launch_near_batch(b->L, cs);
    cudaError_t e2 = cudaStreamEndCapture(cs, &g);
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, g, 0);
    if (g) cudaGraphDestroy(g);
    cudaStreamDestroy(cs);
    if (e != cudaSuccess) {
      b->exec = nullptr;
      return beast_fail(ctx, BEAST_ERR_CUDA, std::string("batch graph: ") + cudaGetErrorString(e));
    }
  }
  {
    ProfScope ps(ctx, PK_FAR, 228.0 * (double)b->L.ntiles * b->L.tile_m * b->L.tile_q, 2);
    BEAST_CUDA_TRY(ctx, cudaGraphLaunch(b->exec, st));
  }
  int h[2] = {0, 0};
  BEAST_CUDA_TRY(ctx, cudaMemcpyAsync(h, b->counter, sizeof(h), cudaMemcpyDeviceToHost, st));
  BEAST_CUDA_TRY(ctx, cudaStreamSynchronize(st));
  if ((h[1] & 1) || h[0] > b->L.near_cap) return beast_fail(ctx, BEAST_ERR_ARG, "batch near-pair list overflow");
  if (h[1] & 2)
    return beast_fail(ctx, BEAST_ERR_UNSUPPORTED, "singularity extraction not available for this operator/space pairing");
  return BEAST_OK;
}

int beast_batch_free(beast_batch* b) {
  if (!b) return BEAST_OK;
  cudaSetDevice(b->ctx->device);
  cudaStreamSynchronize(b->ctx->stream);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  for (void* p : b->zcols) cudaFree(p);
  if (b->jobs) cudaFree(b->jobs);
  if (b->tiles) cudaFree(b->tiles);
  if (b->near) cudaFree(b->near);
  if (b->counter) cudaFree(b->counter);
  delete b;
  return BEAST_OK;
}

int beast_solve_job(beast_ctx* ctx, const beast_op_desc* op, const beast_qs_desc* qs,
                    const beast_space* space, int exc_kind, const double* dir, const double* pol,
                    double egr, double egi, int precision, double tol, double* x, int x_loc,
                    int* iters, double* resid) {
  ARG_CHECK(ctx, ctx && op && qs && space && dir && x, "null argument");
  beast_system* y = nullptr;
  int rc = beast_system_create(ctx, op, qs, space, -1, 0.0, 0.0, precision, &y);
  if (rc) return rc;
  rc = beast_system_solve(ctx, y, exc_kind, 1, dir, pol, egr, egi, tol, x, x_loc, iters, resid);
  beast_system_free(y);
  return rc;
}

}  // extern "C"
