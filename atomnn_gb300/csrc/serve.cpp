// serve.cpp - continuous batching of energy+force requests (nnpgpu_serve_*, include/nnpgpu.h).
//
// The reference's compute tool evaluates a fixed file list (src/nnp/nnpce.cpp:273-281); this
// loop serves the same computation for requests that arrive over time:
//   * requests wait in a FIFO queue; each of K slots (a context with its own stream and device
//     buffers, driven by its own host thread) takes every queued request that fits its atom
//     budget as soon as it is free, so requests that arrive while other batches run on the GPU
//     join the next batch and batches of different slots overlap on the device;
//   * a request larger than a slot's share of the HBM budget is refused at submission;
//   * requests carrying a resident key keep that structure's neighbour list on the device,
//     built with cutoff rc + skin; a later request of the same key whose atoms moved less than
//     skin/2 (same cell and species) re-decides the exact rc list from it instead of searching
//     all atoms (neighbour mode 3).  Resident lists are evicted least-recently-used when they
//     would exceed their share of the budget.  Requests of one key are processed in order.
//   * a keyed request whose positions, species and cell equal (bit for bit) those of the key's
//     last evaluated request is answered at submission from the key's resident results: its
//     descriptors, network outputs and forces would be the same.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <unordered_map>

#include "context.h"

namespace nnpgpu {

namespace {
using Clock = std::chrono::steady_clock;

struct Req {
  long long id = 0, key = -1;
  int natoms = 0;
  std::vector<double> posn, cell;
  std::vector<int> species;
  Clock::time_point t0;
  double energy = 0, latency = 0;
  std::vector<double> force;
  int status = NNPGPU_ERR_BUSY;  // BUSY until done
  std::string err;
};

struct Resident {
  int natoms = 0;
  std::vector<int> species;
  double cell[9];
  std::vector<double> ref;  // positions at which the list was built
  int cap = 0;
  int *d_j = nullptr, *d_code = nullptr, *d_cnt = nullptr;
  float4* d_r = nullptr;
  size_t bytes = 0;
  bool busy = false;
  long long last = 0;
  // the last evaluated request of this key (host copies): inputs and results
  bool has_result = false;
  std::vector<double> res_posn, res_cell, res_force;
  std::vector<int> res_species;
  double res_energy = 0;
};
}  // namespace

struct Serving::Impl {
  nnpgpu_ctx* parent = nullptr;
  nnpgpu_serve_opts opts{};
  std::vector<nnpgpu_ctx*> slots;
  std::vector<std::thread> threads;
  std::mutex mu;
  std::condition_variable cv;
  bool stop = false;
  long long next_id = 1, tick = 0;
  std::deque<Req*> queue;
  std::unordered_map<long long, std::unique_ptr<Req>> reqs;
  std::unordered_map<long long, Resident> res;
  size_t res_bytes = 0, res_budget = 0;
  long long slot_atoms_max = 0;
  int flags = 0;

  ~Impl() {
    {
      std::lock_guard<std::mutex> l(mu);
      stop = true;
    }
    cv.notify_all();
    for (auto& t : threads) t.join();
    cudaSetDevice(parent->device);
    for (auto& kv : res) free_res(kv.second);
    for (nnpgpu_ctx* s : slots) nnpgpu_destroy(s);
  }

  void free_res(Resident& r) {
    if (r.d_j) cudaFree(r.d_j);
    if (r.d_code) cudaFree(r.d_code);
    if (r.d_cnt) cudaFree(r.d_cnt);
    if (r.d_r) cudaFree(r.d_r);
    r.d_j = r.d_code = r.d_cnt = nullptr;
    r.d_r = nullptr;
    res_bytes -= r.bytes;
    r.bytes = 0;
  }

  // bytes of device state one atom needs inside a batch (neighbour slots dominate)
  // (slot index, vector, image code, species: 25 B; per atom coordinates, floors, fixed-point and
  // FP64 forces, counts and the network rows)
  static size_t bytes_per_atom(int cap, int gstride) { return (size_t)cap * 28 + (size_t)gstride * 8 + 200; }

  bool can_use_skin(const Resident& r, const Req& q) const {
    if (!r.d_j || r.natoms != q.natoms || r.species != q.species) return false;
    for (int k = 0; k < 9; ++k)
      if (r.cell[k] != q.cell[k]) return false;
    double mx = 0;
    for (int a = 0; a < q.natoms; ++a) {
      const double dx = q.posn[3 * a] - r.ref[3 * a], dy = q.posn[3 * a + 1] - r.ref[3 * a + 1], dz = q.posn[3 * a + 2] - r.ref[3 * a + 2];
      mx = std::max(mx, dx * dx + dy * dy + dz * dz);
    }
    return std::sqrt(mx) <= 0.5 * opts.skin;
  }

  // (re)build the resident list of q's key on slot context c; called without the lock held
  void build_resident(nnpgpu_ctx* c, Resident& r, const Req& q) {
    const double rcs = c->pot.rc + opts.skin;
    int cap = 0;
    {
      // density estimate as for batch capacities, with the larger cutoff
      const double* R = q.cell.data();
      const double vol = std::fabs(R[0] * (R[4] * R[8] - R[7] * R[5]) - R[3] * (R[1] * R[8] - R[7] * R[2]) + R[6] * (R[1] * R[5] - R[4] * R[2]));
      const double nb = vol > 0 ? q.natoms / vol * 4.0 / 3.0 * M_PI * std::pow(rcs + 0.5, 3) * 1.25 + 16 : q.natoms;
      cap = std::min(1024, (int)std::ceil(nb / 32.0) * 32);
    }
    for (int attempt = 0; attempt < 3; ++attempt) {
      const size_t slots_n = (size_t)q.natoms * cap;
      const size_t bytes = slots_n * (4 + 4 + 16) + (size_t)q.natoms * 4;
      {
        std::lock_guard<std::mutex> l(mu);
        free_res(r);
        // evict least-recently-used idle residents until this one fits its share of the budget
        while (res_bytes + bytes > res_budget) {
          long long victim = -1, oldest = -1;
          for (auto& kv : res)
            if (kv.second.d_j && !kv.second.busy && &kv.second != &r && (oldest < 0 || kv.second.last < oldest)) {
              oldest = kv.second.last;
              victim = kv.first;
            }
          if (victim < 0) break;
          free_res(res[victim]);
        }
        if (res_bytes + bytes > res_budget) return;  // no room: this key stays non-resident
        res_bytes += bytes;
        r.bytes = bytes;
      }
      bool ok = cudaMalloc(&r.d_j, slots_n * 4) == cudaSuccess && cudaMalloc(&r.d_code, slots_n * 4) == cudaSuccess &&
                cudaMalloc(&r.d_r, slots_n * 16) == cudaSuccess && cudaMalloc(&r.d_cnt, (size_t)q.natoms * 4) == cudaSuccess;
      if (!ok) {
        cudaGetLastError();
        std::lock_guard<std::mutex> l(mu);
        free_res(r);
        return;
      }
      int maxc = 0;
      const int rcode = build_skin(c, q.natoms, q.posn.data(), q.cell.data(), rcs, cap, r.d_j, r.d_code, r.d_cnt, r.d_r, &maxc);
      if (rcode == NNPGPU_OK) {
        r.natoms = q.natoms;
        r.species = q.species;
        std::memcpy(r.cell, q.cell.data(), sizeof(r.cell));
        r.ref = q.posn;
        r.cap = cap;
        return;
      }
      std::lock_guard<std::mutex> l(mu);
      free_res(r);
      if (rcode != NNPGPU_ERR_CAPACITY || maxc > 1024) return;
      cap = (maxc + 31) / 32 * 32;
    }
  }

  void worker(int s) {
    nnpgpu_ctx* c = slots[s];
    cudaSetDevice(c->device);
    std::vector<Req*> batch;
    std::vector<int> natoms, species;
    std::vector<double> posn, cell, energy, force;
    std::vector<SkinRef> skins;
    std::vector<char> rebuild;
    for (;;) {
      batch.clear();
      {
        std::unique_lock<std::mutex> l(mu);
        for (;;) {
          if (stop) return;
          // continuous batching: take queued requests in order while they fit; skip keys in flight
          long long atoms = 0;
          for (auto it = queue.begin(); it != queue.end();) {
            Req* q = *it;
            if (q->key >= 0 && res.count(q->key) && res[q->key].busy) {
              ++it;
              continue;
            }
            if (!batch.empty() && atoms + q->natoms > slot_atoms_max) break;
            atoms += q->natoms;
            if (q->key >= 0) {
              Resident& r = res[q->key];
              r.busy = true;
              r.last = ++tick;
            }
            batch.push_back(q);
            it = queue.erase(it);
          }
          if (!batch.empty()) break;
          cv.wait(l);
        }
      }
      // assemble the batch (resident lists are used where they are still valid)
      natoms.clear(); species.clear(); posn.clear(); cell.clear(); skins.clear(); rebuild.clear();
      for (Req* q : batch) {
        natoms.push_back(q->natoms);
        species.insert(species.end(), q->species.begin(), q->species.end());
        posn.insert(posn.end(), q->posn.begin(), q->posn.end());
        cell.insert(cell.end(), q->cell.begin(), q->cell.end());
        SkinRef sk;
        bool rb = false;
        if (q->key >= 0 && opts.skin > 0) {
          Resident* r = nullptr;
          {
            std::lock_guard<std::mutex> l(mu);
            r = &res[q->key];
          }
          if (can_use_skin(*r, *q)) {
            sk.j = r->d_j;
            sk.code = r->d_code;
            sk.cnt = r->d_cnt;
            sk.cap = r->cap;
          } else {
            rb = true;
          }
        }
        skins.push_back(sk);
        rebuild.push_back(rb);
      }
      long long tot = 0;
      for (int n : natoms) tot += n;
      energy.assign(batch.size(), 0.0);
      force.assign((size_t)tot * 3, 0.0);
      const int rcode = compute_host(c, (int)batch.size(), natoms.data(), posn.data(), species.data(), cell.data(),
                                     NNPGPU_ENERGY | NNPGPU_FORCE | NNPGPU_BATCHED | flags, energy.data(), force.data(), nullptr,
                                     skins.data());
      const std::string msg = rcode == NNPGPU_OK ? std::string() : c->err;
      // refresh resident lists of keys that could not reuse theirs
      if (rcode == NNPGPU_OK)
        for (size_t k = 0; k < batch.size(); ++k)
          if (rebuild[k]) {
            Resident* r = nullptr;
            {
              std::lock_guard<std::mutex> l(mu);
              r = &res[batch[k]->key];
            }
            build_resident(c, *r, *batch[k]);
          }
      const auto now = Clock::now();
      {
        std::lock_guard<std::mutex> l(mu);
        size_t off = 0;
        for (size_t k = 0; k < batch.size(); ++k) {
          Req* q = batch[k];
          q->status = rcode;
          q->err = msg;
          if (rcode == NNPGPU_OK) {
            q->energy = energy[k];
            q->force.assign(force.begin() + off, force.begin() + off + 3 * (size_t)q->natoms);
          }
          off += 3 * (size_t)q->natoms;
          q->latency = std::chrono::duration<double>(now - q->t0).count();
          if (q->key >= 0) {
            Resident& r = res[q->key];
            r.busy = false;
            if (rcode == NNPGPU_OK) {
              r.has_result = true;
              r.res_posn = q->posn;
              r.res_cell = q->cell;
              r.res_species = q->species;
              r.res_energy = q->energy;
              r.res_force = q->force;
            }
          }
        }
      }
      cv.notify_all();
    }
  }
};

Serving::Serving(nnpgpu_ctx* c, const nnpgpu_serve_opts& o) : impl_(new Impl) {
  Impl& I = *impl_;
  I.parent = c;
  I.opts = o;
  if (I.opts.max_inflight < 1) I.opts.max_inflight = 2;
  if (I.opts.max_inflight > 8) I.opts.max_inflight = 8;
  size_t budget = o.hbm_budget_bytes ? o.hbm_budget_bytes : (c->budget ? c->budget : (size_t)40 << 30);
  I.res_budget = budget / 5;  // resident lists
  const size_t slot_budget = (budget - I.res_budget) / I.opts.max_inflight;
  const size_t per_atom = Impl::bytes_per_atom(256, c->gstride);
  I.slot_atoms_max = (long long)std::min<size_t>(slot_budget / per_atom, (size_t)1 << 22);
  if (o.max_batch_atoms > 0) I.slot_atoms_max = std::min<long long>(I.slot_atoms_max, o.max_batch_atoms);
  I.flags = o.flags & (NNPGPU_BF16 | NNPGPU_NO_VACUUM);
  for (int s = 0; s < I.opts.max_inflight; ++s) {
    nnpgpu_opts so{c->device, c->cap_hint, slot_budget, 0};
    nnpgpu_ctx* sc = nullptr;
    const int rc = nnpgpu_create(c->potfile.c_str(), &so, &sc);
    if (rc != NNPGPU_OK) {
      if (sc) nnpgpu_destroy(sc);
      throw PotError(rc, "could not create a serving slot");
    }
    sc->tune = c->tune;  // slots run with the owner's (possibly autotuned) launch shapes
    I.slots.push_back(sc);
  }
  for (int s = 0; s < I.opts.max_inflight; ++s) I.threads.emplace_back([this, s] { impl_->worker(s); });
}

Serving::~Serving() { delete impl_; }

int Serving::submit(int natoms, const double* posn, const int* species, const double* cell, long long key, long long* id) {
  Impl& I = *impl_;
  if (natoms <= 0 || !posn || !species || !cell || !id) return NNPGPU_ERR_INVALID;
  for (int a = 0; a < natoms; ++a)
    if (species[a] < 0 || species[a] >= I.parent->pot.ntypes) return NNPGPU_ERR_INVALID;
  if (natoms > I.slot_atoms_max) return NNPGPU_ERR_OOM;  // admission: larger than a slot's device budget
  auto q = std::make_unique<Req>();
  q->natoms = natoms;
  q->key = key;
  q->posn.assign(posn, posn + 3 * (size_t)natoms);
  q->species.assign(species, species + natoms);
  q->cell.assign(cell, cell + 9);
  q->t0 = Clock::now();
  {
    std::lock_guard<std::mutex> l(I.mu);
    q->id = I.next_id++;
    *id = q->id;
    auto it = key >= 0 ? I.res.find(key) : I.res.end();
    if (it != I.res.end() && it->second.has_result && it->second.res_posn == q->posn && it->second.res_species == q->species &&
        it->second.res_cell == q->cell) {
      // unchanged inputs: the key's resident results are this request's results
      q->energy = it->second.res_energy;
      q->force = it->second.res_force;
      q->status = NNPGPU_OK;
      q->latency = std::chrono::duration<double>(Clock::now() - q->t0).count();
      it->second.last = ++I.tick;
      I.reqs[q->id] = std::move(q);
      return NNPGPU_OK;
    }
    I.queue.push_back(q.get());
    I.reqs[q->id] = std::move(q);
  }
  I.cv.notify_all();
  return NNPGPU_OK;
}

int Serving::poll(long long id, double* energy, double* force, double* latency) {
  Impl& I = *impl_;
  std::lock_guard<std::mutex> l(I.mu);
  auto it = I.reqs.find(id);
  if (it == I.reqs.end()) return NNPGPU_ERR_INVALID;
  Req& q = *it->second;
  if (q.status == NNPGPU_ERR_BUSY) return NNPGPU_ERR_BUSY;
  const int st = q.status;
  if (st == NNPGPU_OK) {
    if (energy) *energy = q.energy;
    if (force) std::memcpy(force, q.force.data(), sizeof(double) * q.force.size());
  } else {
    I.parent->err = q.err;
  }
  if (latency) *latency = q.latency;
  I.reqs.erase(it);
  return st;
}

}  // namespace nnpgpu

using namespace nnpgpu;

extern "C" int nnpgpu_serve_start(nnpgpu_ctx* c, const nnpgpu_serve_opts* opts) {
  if (!c || !c->stream) return set_error(c, NNPGPU_ERR_CUDA, "context has no device");
  if (c->serving) return set_error(c, NNPGPU_ERR_INVALID, "serving already started");
  nnpgpu_serve_opts o{};
  if (opts) o = *opts;
  if (o.skin < 0) return set_error(c, NNPGPU_ERR_INVALID, "negative skin");
  try {
    c->serving.reset(new Serving(c, o));
  } catch (PotError& e) {
    return set_error(c, e.code, e.what());
  }
  return NNPGPU_OK;
}

extern "C" int nnpgpu_submit(nnpgpu_ctx* c, int natoms, const double* posn, const int* species, const double* cell,
                             long long resident_key, long long* request_id) {
  if (!c || !c->serving) return set_error(c, NNPGPU_ERR_INVALID, "serving not started");
  const int rc = c->serving->submit(natoms, posn, species, cell, resident_key, request_id);
  if (rc == NNPGPU_ERR_OOM) return set_error(c, rc, "request larger than the device budget of a serving slot");
  if (rc != NNPGPU_OK) return set_error(c, rc, "invalid request");
  return NNPGPU_OK;
}

extern "C" int nnpgpu_poll(nnpgpu_ctx* c, long long request_id, double* energy, double* force, double* latency_s) {
  if (!c || !c->serving) return set_error(c, NNPGPU_ERR_INVALID, "serving not started");
  return c->serving->poll(request_id, energy, force, latency_s);
}

extern "C" int nnpgpu_serve_stop(nnpgpu_ctx* c) {
  if (!c || !c->serving) return set_error(c, NNPGPU_ERR_INVALID, "serving not started");
  c->serving.reset();
  return NNPGPU_OK;
}
