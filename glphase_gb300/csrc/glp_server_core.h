// glp_server_core.h -- the scheduling of the request server (glp_server_*),
// free of CUDA so that it compiles and is tested on any host.
//
// Requests (a problem handle, a generation template, a generation count) wait
// in arrival order.  A tick admits waiting requests while their device
// footprint fits the budget, hands the launcher one generation of every
// resident request grouped into launches -- all requests of one emission
// source in one launch, or one launch per request in the plain form -- and,
// when the launcher succeeds, advances every resident request by one
// generation and retires those that have run all of theirs.  A request's
// generation g takes the template with generation = g; pen = min((g+1)/B,
// 1)^2 in binary32 for a burn-in B > 0 (Insti::estimate, insti.cpp:1670-1671);
// haps and hnew exchanged on odd g; the kick-start range in g = 0 only.
#ifndef GLP_SERVER_CORE_H
#define GLP_SERVER_CORE_H

#include <algorithm>
#include <cstdint>
#include <deque>
#include <unordered_map>
#include <utility>
#include <vector>

#include "../../include/glphase_gpu.h"

namespace glp {

struct ServerCore {
  struct Req {
    uint64_t id = 0;
    void *problem = nullptr;
    glp_generation_args tmpl{};
    uint32_t generations = 0, gen = 0;
    uint64_t bytes = 0;
    int state = GLP_REQ_QUEUED;
  };
  // one launch: the problems and their generation arguments
  struct Launch {
    std::vector<void *> problems;
    std::vector<glp_generation_args> args;
  };

  uint64_t budget = 0, used = 0;
  bool plain = false;
  uint64_t next_id = 1, ticks = 0, updates = 0;
  std::unordered_map<uint64_t, Req> reqs;
  std::deque<uint64_t> queue;    // waiting, in arrival order
  std::vector<uint64_t> active;  // resident, in admission order

  // Device bytes a request holds while resident: emission, genotype
  // probabilities, hmm_work scratch, both haplotype buffers.
  static uint64_t footprint(const glp_generation_args &a) {
    const uint64_t N = a.num_samples, S = a.num_sites, H = a.num_haps;
    return N * S * (16 + 12 + 16) + 2 * H * ((S + 63) / 64) * 8;
  }

  // The arguments of a request's next generation.
  static glp_generation_args args_of(const Req &r) {
    glp_generation_args a = r.tmpl;
    const uint32_t g = r.gen;
    a.generation = g;
    if (r.tmpl.burnin) {
      const float x = std::min((float)(g + 1u) / (float)r.tmpl.burnin, 1.0f);
      a.pen = x * x;
    }
    if (g & 1u) {
      a.haps = r.tmpl.hnew;
      a.hnew = const_cast<uint64_t *>(r.tmpl.haps);
    }
    if (r.tmpl.kick_start && g > 0) {
      a.kick_start = 0;
      a.sample_lo = a.sample_hi = 0;
    }
    return a;
  }

  // A request as it would be queued (not yet added): for validation.
  static Req make(void *problem, const glp_generation_args &tmpl, uint32_t generations) {
    Req r;
    r.problem = problem;
    r.tmpl = tmpl;
    r.generations = generations;
    r.bytes = footprint(tmpl);
    return r;
  }

  uint64_t add(Req r) {
    r.id = next_id++;
    r.state = GLP_REQ_QUEUED;
    r.gen = 0;
    const uint64_t id = r.id;
    reqs.emplace(id, r);
    queue.push_back(id);
    return id;
  }

  // Admit in arrival order while the next waiting request fits.
  void admit() {
    while (!queue.empty()) {
      Req &r = reqs.at(queue.front());
      if (used + r.bytes > budget)
        break;
      used += r.bytes;
      r.state = GLP_REQ_RESIDENT;
      active.push_back(r.id);
      queue.pop_front();
    }
  }

  // The launches of one generation of every resident request.
  std::vector<Launch> launches() const {
    std::vector<Launch> out;
    if (plain) {
      for (uint64_t id : active) {
        const Req &r = reqs.at(id);
        out.push_back(Launch{{r.problem}, {args_of(r)}});
      }
      return out;
    }
    for (uint32_t vq = 0; vq < 2; ++vq) {  // a launch holds one emission source
      Launch l;
      for (uint64_t id : active) {
        const Req &r = reqs.at(id);
        if (((r.tmpl.flags & GLP_GEN_VQ) != 0) == (vq == 1)) {
          l.problems.push_back(r.problem);
          l.args.push_back(args_of(r));
        }
      }
      if (!l.problems.empty())
        out.push_back(std::move(l));
    }
    return out;
  }

  // Admit, run `run(launches)` (returns a status; 0 = done on the device),
  // then advance and retire.  On a failed run nothing advances.
  template <class Run>
  int tick(Run &&run, uint32_t *resident, uint32_t *finished) {
    admit();
    if (resident)
      *resident = (uint32_t)active.size();
    if (finished)
      *finished = 0;
    if (active.empty())
      return 0;
    const int rc = run(launches());
    if (rc)
      return rc;
    ++ticks;
    uint32_t done = 0;
    std::vector<uint64_t> still;
    for (uint64_t id : active) {
      Req &r = reqs.at(id);
      updates += (uint64_t)r.tmpl.num_samples * (r.tmpl.num_cycles + 1) * r.tmpl.num_sites;
      if (++r.gen >= r.generations) {
        r.state = GLP_REQ_DONE;
        used -= r.bytes;
        ++done;
      } else {
        still.push_back(id);
      }
    }
    active.swap(still);
    if (finished)
      *finished = done;
    return 0;
  }

  const Req *find(uint64_t id) const {
    auto it = reqs.find(id);
    return it == reqs.end() ? nullptr : &it->second;
  }

  // The buffer holding a request's current haplotypes.
  static const uint64_t *current_haps(const Req &r) {
    return (r.gen & 1u) ? r.tmpl.hnew : r.tmpl.haps;
  }

  // Forget a finished request: 0, or 1 when unknown, 2 when not finished.
  int release(uint64_t id) {
    auto it = reqs.find(id);
    if (it == reqs.end())
      return 1;
    if (it->second.state != GLP_REQ_DONE)
      return 2;
    reqs.erase(it);
    return 0;
  }
};

}  // namespace glp

#endif  // GLP_SERVER_CORE_H
