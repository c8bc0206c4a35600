// Serving engine: continuous batching of variational circuit jobs on one GPU.
//
// A client is a VQE / Trotter loop of the reference (variational_apply followed
// by expect(state, H); BlueTangle.jl src/vqa.jl:420-456, src/func.jl:100): a
// fixed circuit, compiled once (a plan, or a program for trajectory batches),
// evaluated again and again at new parameters, each time returning <H> of a
// Pauli sum.  The engine
//   * keeps each client's state resident between its requests and admits clients
//     by HBM footprint, evicting idle residents least-recently-used first and
//     holding a request back while nothing can be evicted;
//   * runs requests on `lanes` host threads, each with its own context (CUDA
//     stream), so requests arriving while others are on the GPU start as soon as a
//     lane is free and their kernels overlap on the device;
//   * serves a client's requests in arrival order (they share its state), one at
//     a time, on the lane its state lives on;
//   * packs small circuits into one launch: a packed client is a program whose
//     members are independent requests, so up to its width of queued requests run
//     as one shared-memory program launch (one CTA per request);
//   * runs the queued requests of a plan client whose state is too small to fill
//     the GPU (fewer than 2^22 amplitudes) together: its resident state holds
//     2^(22-n) members (at most 8), and up to that many requests naming the same
//     gates run as one plan run over the members, each with its own matrices
//     (bt_plan_run_members: the passes holding those gates read per-member
//     entries, the others launch once for all);
//   * records submit-to-done latency per request for p50/p99.
// A request carries new matrices for some of the client's gates (plan add
// indices, or program op indices) and a seed for the program's draws.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "bt_internal.cuh"

namespace {

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct Req {
  int64_t ticket = 0, client = 0;
  std::vector<int64_t> idx;
  std::vector<double> mats;
  uint64_t seed = 0;
  double t_submit = 0, t_start = 0, t_done = 0;
  double value = 0;
  int status = 0;
  std::string err;
  bool done = false;
};

struct Client {
  int64_t id = 0;
  bt_plan* plan = nullptr;
  bt_program* prog = nullptr;
  int repr = 0, prec = 0, n = 0, batch = 1;
  std::vector<uint64_t> x, z;
  std::vector<double> coef;
  std::vector<int> gate_dim;  // program: matrix dimension of each op (0: not a gate)
  // packed client: a program whose members are independent requests (one per
  // member, its own matrices for the per-member gates); up to `batch` queued
  // requests naming the same gates run in one launch
  bool packed = false;
  std::vector<char> per_member;
  int width = 1;  // plan client: requests per plan run (members of its state)
  size_t footprint = 0;
  bt_state* state = nullptr;  // resident state (nullptr: not resident)
  bool reserved = false;      // admitted, state being allocated by `lane`
  int lane = -1;
  bool busy = false;
  double last_used = 0;
  std::deque<Req*> queue;
};

}  // namespace

struct bt_server {
  int device = 0;
  size_t budget = 0, used = 0;
  std::vector<bt_ctx*> lanes;
  std::vector<std::thread> threads;
  std::mutex mu;
  std::condition_variable cv;
  bool stop = false;
  std::map<int64_t, Client*> clients;
  std::map<int64_t, Req*> reqs;
  int64_t next_client = 0, next_ticket = 0;
  // latencies of the most recent requests (a ring of kLatWindow) for p50/p99;
  // a long-running server keeps a bounded window, not every request
  static constexpr size_t kLatWindow = 65536;
  std::vector<double> latencies;
  size_t lat_next = 0;
  int64_t completed = 0;
  int64_t runs = 0;  // request launches (a packed run serves several requests)
  std::string err;
};

// program/plan hooks (bt_program.cu, bt_plan.cu)
int bt_program_gate_dims(const bt_program* p, std::vector<int>& dims, int* n, int* prec, int* batch,
                         std::vector<char>* per_member);
int bt_plan_shape(const bt_plan* p, int* n, int* repr, int* prec);
int bt_plan_variable_adds(const bt_plan* p, std::vector<int64_t>& idx);
int bt_plan_gate_dims(const bt_plan* p, const int64_t* idx, int count, size_t* reals);

static Client* pick(bt_server* s, int lane) {
  Client* best = nullptr;
  for (auto& kv : s->clients) {
    Client* c = kv.second;
    if (c->queue.empty() || c->busy) continue;
    if ((c->state || c->reserved) && c->lane != lane) continue;  // resident on another lane
    if (!best || c->queue.front()->t_submit < best->queue.front()->t_submit) best = c;
  }
  return best;
}

// reserves HBM for c on `lane`, evicting idle residents LRU-first; false: wait
static bool admit(bt_server* s, Client* c, int lane, std::vector<bt_state*>& to_free) {
  if (c->footprint > s->budget) return false;
  while (s->used + c->footprint > s->budget) {
    Client* victim = nullptr;
    for (auto& kv : s->clients) {
      Client* o = kv.second;
      if (o->state && !o->busy && (!victim || o->last_used < victim->last_used)) victim = o;
    }
    if (!victim) return false;
    to_free.push_back(victim->state);
    victim->state = nullptr;
    victim->lane = -1;
    s->used -= victim->footprint;
  }
  s->used += c->footprint;
  c->reserved = true;
  c->lane = lane;
  return true;
}

// <H> / norm of member m of the client's state
static int member_value(Client* c, int64_t m, double* value) {
  const int nt = (int)c->coef.size();
  std::vector<double> ev(nt);
  double nrm = 0;
  int rc = nt ? bt_expect_pauli(c->state, nt, c->x.data(), c->z.data(), c->coef.data(), m, ev.data()) : BT_OK;
  if (!rc) rc = bt_norm2(c->state, m, &nrm);
  if (rc) return rc;
  double h = 0;
  for (int t = 0; t < nt; ++t) h += ev[t];
  *value = h / nrm;
  return BT_OK;
}

// requests rs of a plan client: one request on member 0 with the plan's own
// matrices; several (all naming the same gates) as one run over members
// [0, k), member m with request m's matrices
static int run_plan(Client* c, const std::vector<Req*>& rs, std::vector<double>& values) {
  const int k = (int)rs.size();
  values.assign(k, 0.0);
  int rc = BT_OK;
  if (k == 1 || rs[0]->idx.empty()) {
    for (int i = 0; i < k && !rc; ++i) {
      if (!rs[i]->idx.empty())
        rc = bt_plan_set_matrices(c->plan, (int)rs[i]->idx.size(), rs[i]->idx.data(), rs[i]->mats.data());
      if (!rc) rc = bt_state_set_zero(c->state, 0);
      if (!rc) rc = bt_plan_run(c->plan, c->state, 0);
      if (!rc) rc = member_value(c, 0, &values[i]);
    }
    return rc;
  }
  std::vector<double> mats;
  for (Req* r : rs) mats.insert(mats.end(), r->mats.begin(), r->mats.end());
  for (int m = 0; m < k && !rc; ++m) rc = bt_state_set_zero(c->state, m);
  if (!rc)
    rc = bt_plan_run_members_n(c->plan, c->state, k, (int)rs[0]->idx.size(), rs[0]->idx.data(), mats.data());
  for (int m = 0; m < k && !rc; ++m) rc = member_value(c, m, &values[m]);
  return rc;
}

static int run_request(bt_ctx* ctx, Client* c, Req* r, double* value) {
  int rc = BT_OK;
  {
    size_t off = 0;
    for (size_t i = 0; i < r->idx.size() && !rc; ++i) {
      const int64_t oi = r->idx[i];
      const int d = oi >= 0 && oi < (int64_t)c->gate_dim.size() ? c->gate_dim[oi] : 0;
      if (!d) return bt_fail(ctx, BT_ERR_BAD_ARG, "request names an op that is not a gate of the program");
      rc = bt_program_set_gate(c->prog, oi, r->mats.data() + off);
      off += (size_t)2 * d * d;
    }
    if (!rc) rc = bt_state_set_zero(c->state, -1);
    if (!rc) rc = bt_program_run(c->prog, c->state, nullptr, r->seed, nullptr);
  }
  if (rc) return rc;
  // <H> per member divided by the member's norm (trace), averaged over members
  const int nt = (int)c->coef.size();
  std::vector<double> ev((size_t)c->batch * nt), nrm(c->batch);
  if (nt) rc = bt_expect_pauli(c->state, nt, c->x.data(), c->z.data(), c->coef.data(), -1, ev.data());
  if (!rc) rc = bt_norm2(c->state, -1, nrm.data());
  if (rc) return rc;
  double acc = 0;
  for (int m = 0; m < c->batch; ++m) {
    double h = 0;
    for (int t = 0; t < nt; ++t) h += ev[(size_t)m * nt + t];
    acc += h / nrm[m];
  }
  *value = acc / c->batch;
  return BT_OK;
}

// requests rs (1 <= size <= batch, all naming the same gates) of a packed client
// as the members of one program run: member m takes request m's matrices (the
// members past the last request repeat it), <H> / norm of member m is request
// m's value
static int run_packed(Client* c, const std::vector<Req*>& rs, std::vector<double>& values) {
  const int K = c->batch, k = (int)rs.size();
  const std::vector<int64_t>& idx = rs[0]->idx;
  std::vector<size_t> off(k, 0);
  std::vector<double> mats;
  int rc = BT_OK;
  for (size_t i = 0; i < idx.size() && !rc; ++i) {
    const int d = c->gate_dim[idx[i]];
    const size_t sz = (size_t)2 * d * d;
    mats.resize(sz * K);
    for (int m = 0; m < K; ++m) {
      const int r = m < k ? m : k - 1;
      memcpy(&mats[sz * m], rs[r]->mats.data() + off[r], sz * sizeof(double));
    }
    for (int r = 0; r < k; ++r) off[r] += sz;
    rc = bt_program_set_gate(c->prog, idx[i], mats.data());
  }
  if (!rc) rc = bt_state_set_zero(c->state, -1);
  if (!rc) rc = bt_program_run(c->prog, c->state, nullptr, rs[0]->seed, nullptr);
  if (rc) return rc;
  const int nt = (int)c->coef.size();
  std::vector<double> ev((size_t)K * nt), nrm(K);
  if (nt) rc = bt_expect_pauli(c->state, nt, c->x.data(), c->z.data(), c->coef.data(), -1, ev.data());
  if (!rc) rc = bt_norm2(c->state, -1, nrm.data());
  if (rc) return rc;
  values.assign(k, 0.0);
  for (int m = 0; m < k; ++m) {
    double h = 0;
    for (int t = 0; t < nt; ++t) h += ev[(size_t)m * nt + t];
    values[m] = h / nrm[m];
  }
  return BT_OK;
}

static void worker(bt_server* s, int lane) {
  bt_ctx* ctx = s->lanes[lane];
  for (;;) {
    Client* c = nullptr;
    std::vector<Req*> rs;
    std::vector<bt_state*> to_free;
    bool alloc = false;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      for (;;) {
        if (s->stop) return;
        c = pick(s, lane);
        if (c && (c->state || c->reserved || admit(s, c, lane, to_free))) break;
        c = nullptr;
        s->cv.wait_for(lk, std::chrono::milliseconds(5));
      }
      c->busy = true;
      alloc = c->state == nullptr;
      rs.push_back(c->queue.front());
      c->queue.pop_front();
      // a packed client (and a plan client of several members) takes the queued
      // requests that name the same gates, up to its width
      const int width = c->packed ? c->batch : (c->plan ? c->width : 1);
      while ((int)rs.size() < width && !c->queue.empty() && c->queue.front()->idx == rs[0]->idx) {
        rs.push_back(c->queue.front());
        c->queue.pop_front();
      }
    }
    for (bt_state* st : to_free) bt_state_free(st);
    int rc = BT_OK;
    if (alloc) {
      bt_state* st = nullptr;
      rc = bt_state_alloc(ctx, c->n, c->repr, c->prec, c->batch, &st);
      std::lock_guard<std::mutex> lk(s->mu);
      c->reserved = false;
      if (rc) {  // give the reservation back
        s->used -= c->footprint;
        c->lane = -1;
      } else {
        c->state = st;
      }
    }
    const double t0 = now_s();
    std::vector<double> v(rs.size(), 0.0);
    if (!rc) rc = c->packed ? run_packed(c, rs, v) : (c->plan ? run_plan(c, rs, v) : run_request(ctx, c, rs[0], &v[0]));
    const double t = now_s();
    std::string err;
    if (rc) err = bt_last_error(nullptr);  // every failure also lands in this thread's message
    std::lock_guard<std::mutex> lk(s->mu);
    for (size_t i = 0; i < rs.size(); ++i) {
      Req* r = rs[i];
      r->t_start = t0;
      r->value = v[i];
      r->status = rc;
      r->err = err;
      r->t_done = t;
      r->done = true;
      if (s->latencies.size() < bt_server::kLatWindow) s->latencies.push_back(t - r->t_submit);
      else s->latencies[s->lat_next] = t - r->t_submit;
      s->lat_next = (s->lat_next + 1) % bt_server::kLatWindow;
      ++s->completed;
    }
    ++s->runs;
    c->busy = false;
    c->last_used = t;
    s->cv.notify_all();
  }
}

static int add_client(bt_server* s, Client* c, int nterms, const uint64_t* x, const uint64_t* z, const double* coef,
                      int64_t* id) {
  if (nterms < 0 || (nterms > 0 && (!x || !z))) {
    delete c;
    return bt_fail(nullptr, BT_ERR_BAD_ARG, "bad Pauli term arrays");
  }
  c->x.assign(x, x + nterms);
  c->z.assign(z, z + nterms);
  c->coef.resize(nterms);
  for (int t = 0; t < nterms; ++t) c->coef[t] = coef ? coef[t] : 1.0;
  const size_t es = c->prec == BT_PREC_C64 ? 8 : 16;
  c->footprint = ((size_t)1 << (c->repr == BT_REPR_DM ? 2 * c->n : c->n)) * es * c->batch;
  std::lock_guard<std::mutex> lk(s->mu);
  c->id = s->next_client++;
  s->clients[c->id] = c;
  if (id) *id = c->id;
  return BT_OK;
}

extern "C" {

int bt_serve_create(int device, int lanes, uint64_t seed, uint64_t hbm_budget, bt_server** out) {
  if (!out || lanes < 1 || lanes > 64) return bt_fail(nullptr, BT_ERR_BAD_ARG, "need 1..64 lanes and an out pointer");
  *out = nullptr;
  bt_server* s = new bt_server();
  s->device = device;
  s->budget = hbm_budget ? hbm_budget : ((uint64_t)200 << 30);
  for (int i = 0; i < lanes; ++i) {
    bt_ctx* c = nullptr;
    // one key for every lane: a request's draws depend on its seed, not on its lane
    int rc = bt_ctx_create(device, seed, &c);
    if (rc) {
      for (bt_ctx* o : s->lanes) bt_ctx_destroy(o);
      delete s;
      return rc;
    }
    s->lanes.push_back(c);
  }
  for (int i = 0; i < lanes; ++i) s->threads.emplace_back(worker, s, i);
  *out = s;
  return BT_OK;
}

int bt_serve_destroy(bt_server* s) {
  if (!s) return BT_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    s->cv.notify_all();
  }
  for (auto& t : s->threads) t.join();
  for (auto& kv : s->clients) {
    if (kv.second->state) bt_state_free(kv.second->state);
    delete kv.second;
  }
  for (auto& kv : s->reqs) delete kv.second;  // queued requests are owned here
  for (bt_ctx* c : s->lanes) bt_ctx_destroy(c);
  delete s;
  return BT_OK;
}

int bt_serve_add_plan_client(bt_server* s, bt_plan* plan, int nterms, const uint64_t* xmask, const uint64_t* zmask,
                             const double* coef, int64_t* client) {
  if (!s || !plan) return bt_fail(nullptr, BT_ERR_BAD_ARG, "NULL server or plan");
  Client* c = new Client();
  c->plan = plan;
  int rc = bt_plan_shape(plan, &c->n, &c->repr, &c->prec);
  if (rc) {
    delete c;
    return rc;
  }
  // a state vector of fewer than 2^22 amplitudes leaves most SMs idle: hold up to
  // 8 requests' members, so that queued requests run together; the per-member
  // kernels of the variable gates are built now rather than at the first such run
  if (c->repr == BT_REPR_SV && c->n < 22) {
    std::vector<int64_t> var;
    if (!bt_plan_variable_adds(plan, var) && !var.empty() &&
        !bt_plan_prepare_members(plan, (int)var.size(), var.data()))
      c->width = std::min(8, 1 << (22 - c->n));
    // within the server's HBM budget, or the client could never be admitted
    const size_t member = ((size_t)1 << c->n) * (c->prec == BT_PREC_C64 ? 8 : 16);
    while (c->width > 1 && member * c->width > s->budget) c->width /= 2;
  }
  c->batch = c->width;
  return add_client(s, c, nterms, xmask, zmask, coef, client);
}

int bt_serve_add_program_client(bt_server* s, bt_program* prog, int nterms, const uint64_t* xmask,
                                const uint64_t* zmask, const double* coef, int64_t* client) {
  if (!s || !prog) return bt_fail(nullptr, BT_ERR_BAD_ARG, "NULL server or program");
  Client* c = new Client();
  c->prog = prog;
  c->repr = BT_REPR_SV;
  int rc = bt_program_gate_dims(prog, c->gate_dim, &c->n, &c->prec, &c->batch, &c->per_member);
  if (rc) {
    delete c;
    return rc;
  }
  return add_client(s, c, nterms, xmask, zmask, coef, client);
}

int bt_serve_add_packed_client(bt_server* s, bt_program* prog, int nterms, const uint64_t* xmask,
                               const uint64_t* zmask, const double* coef, int64_t* client) {
  if (!s || !prog) return bt_fail(nullptr, BT_ERR_BAD_ARG, "NULL server or program");
  Client* c = new Client();
  c->prog = prog;
  c->repr = BT_REPR_SV;
  c->packed = true;
  int rc = bt_program_gate_dims(prog, c->gate_dim, &c->n, &c->prec, &c->batch, &c->per_member);
  if (rc) {
    delete c;
    return rc;
  }
  return add_client(s, c, nterms, xmask, zmask, coef, client);
}

int bt_serve_submit(bt_server* s, int64_t client, int count, const int64_t* index, const double* mats, uint64_t seed,
                    int64_t* ticket) {
  if (!s || !ticket) return bt_fail(nullptr, BT_ERR_BAD_ARG, "NULL server or ticket");
  if (count < 0 || (count > 0 && (!index || !mats))) return bt_fail(nullptr, BT_ERR_BAD_ARG, "bad matrix update arrays");
  Req* r = new Req();
  r->client = client;
  r->seed = seed;
  r->idx.assign(index, index + count);
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->clients.find(client);
  if (it == s->clients.end()) {
    delete r;
    return bt_fail(nullptr, BT_ERR_BAD_ARG, "unknown client");
  }
  Client* c = it->second;
  if (c->footprint > s->budget) {
    delete r;
    return bt_fail(nullptr, BT_ERR_OOM, "the client's state is larger than the server's HBM budget");
  }
  // matrices back to back in each gate's size (the size each gate was added with)
  size_t reals = 0;
  if (c->plan) {
    int rc = bt_plan_gate_dims(c->plan, r->idx.data(), count, &reals);
    if (rc) {
      delete r;
      return rc;
    }
  } else {
    for (int i = 0; i < count; ++i) {
      const int64_t oi = index[i];
      const int d = oi >= 0 && oi < (int64_t)c->gate_dim.size() ? c->gate_dim[oi] : 0;
      if (!d) {
        delete r;
        return bt_fail(nullptr, BT_ERR_BAD_ARG, "index names an op that is not a gate of the program");
      }
      if (c->packed && !c->per_member[oi]) {
        delete r;
        return bt_fail(nullptr, BT_ERR_BAD_ARG, "a packed client's request names a gate without per-member matrices");
      }
      reals += (size_t)2 * d * d;
    }
  }
  r->mats.assign(mats, mats + reals);
  r->ticket = s->next_ticket++;
  r->t_submit = now_s();
  s->reqs[r->ticket] = r;
  c->queue.push_back(r);
  *ticket = r->ticket;
  s->cv.notify_all();
  return BT_OK;
}

int bt_serve_poll(bt_server* s, int64_t ticket, int64_t wait_ms, double* value, double* latency_s,
                  double* service_s) {
  if (!s) return bt_fail(nullptr, BT_ERR_BAD_ARG, "server is NULL");
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return bt_fail(nullptr, BT_ERR_BAD_ARG, "unknown ticket");
  Req* r = it->second;
  if (!r->done && wait_ms != 0) {
    auto pred = [&] { return r->done; };
    if (wait_ms < 0) s->cv.wait(lk, pred);
    else s->cv.wait_for(lk, std::chrono::milliseconds(wait_ms), pred);
  }
  if (!r->done) return BT_ERR_TIMEOUT;
  if (value) *value = r->value;
  if (latency_s) *latency_s = r->t_done - r->t_submit;
  if (service_s) *service_s = r->t_done - r->t_start;
  int st = r->status;
  if (st) bt_fail(nullptr, st, r->err);
  s->reqs.erase(it);
  delete r;
  return st;
}

int bt_serve_stats(bt_server* s, int64_t* completed, double* p50_s, double* p99_s, int64_t* resident,
                   uint64_t* hbm_used, int64_t* runs) {
  if (!s) return bt_fail(nullptr, BT_ERR_BAD_ARG, "server is NULL");
  std::lock_guard<std::mutex> lk(s->mu);
  std::vector<double> l = s->latencies;
  std::sort(l.begin(), l.end());
  auto pct = [&](double q) {
    if (l.empty()) return 0.0;
    const double pos = q * (double)(l.size() - 1);
    const size_t i = (size_t)pos;
    const double f = pos - (double)i;
    return i + 1 < l.size() ? l[i] * (1 - f) + l[i + 1] * f : l[i];
  };
  if (completed) *completed = s->completed;
  if (p50_s) *p50_s = pct(0.50);
  if (p99_s) *p99_s = pct(0.99);
  int64_t res = 0;
  for (auto& kv : s->clients) res += kv.second->state != nullptr;
  if (resident) *resident = res;
  if (hbm_used) *hbm_used = s->used;
  if (runs) *runs = s->runs;
  return BT_OK;
}

}  // extern "C"
