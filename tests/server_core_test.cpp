// Host logic of the request server's scheduling (glp_server_core.h) with a
// fake launcher: admission under the budget in arrival order, per-request
// generation arguments, launch grouping, retirement, release.  Built and run
// by tests/test_server_core.py with the host C++ compiler; no GPU.
#include <cstdio>
#include <cstring>

#include "../glphase_gb300/csrc/glp_server_core.h"

static int failures = 0;
#define CHECK(cond)                                                  \
  do {                                                               \
    if (!(cond)) {                                                   \
      std::printf("FAIL %s:%d: %s\n", __FILE__, __LINE__, #cond);    \
      ++failures;                                                    \
    }                                                                \
  } while (0)

using glp::ServerCore;

static uint64_t bufs[64][2];

static glp_generation_args tmpl(uint32_t N, uint32_t S, uint32_t C, int k, uint32_t burnin = 0,
                                uint32_t flags = 0) {
  glp_generation_args a;
  std::memset(&a, 0, sizeof(a));
  a.num_samples = N;
  a.num_sites = S;
  a.num_cycles = C;
  a.num_haps = 2 * N;
  a.haps = &bufs[k][0];
  a.hnew = &bufs[k][1];
  a.pen = 0.5f;
  a.seed = 100 + k;
  a.burnin = burnin;
  a.flags = flags;
  return a;
}

static void *problem(int k) { return &bufs[k][0] + 1000; }

int main() {
  // footprint: emission, genotype probabilities, scratch, two haplotype buffers
  CHECK(ServerCore::footprint(tmpl(100, 640, 10, 0)) == 100ull * 640 * 44 + 2ull * 200 * 10 * 8);

  // generation arguments
  {
    ServerCore::Req r = ServerCore::make(problem(1), tmpl(4, 64, 5, 1, 3), 6);
    const float want[6] = {(1.0f / 3) * (1.0f / 3), (2.0f / 3) * (2.0f / 3), 1, 1, 1, 1};
    for (uint32_t g = 0; g < 6; ++g) {
      r.gen = g;
      const glp_generation_args a = ServerCore::args_of(r);
      const float x = std::min((float)(g + 1) / 3.0f, 1.0f);
      CHECK(a.generation == g && a.pen == x * x && a.pen == want[g]);
      CHECK(a.haps == ((g & 1) ? &bufs[1][1] : &bufs[1][0]));
      CHECK(a.hnew == ((g & 1) ? &bufs[1][0] : &bufs[1][1]));
      CHECK(ServerCore::current_haps(r) == a.haps);
    }
    ServerCore::Req q = ServerCore::make(problem(2), tmpl(4, 64, 5, 2), 2);
    q.tmpl.kick_start = 1;
    q.tmpl.sample_lo = 8;
    q.tmpl.sample_hi = 20;
    glp_generation_args a0 = ServerCore::args_of(q);
    CHECK(a0.pen == 0.5f && a0.kick_start == 1 && a0.sample_lo == 8 && a0.sample_hi == 20);
    q.gen = 1;
    glp_generation_args a1 = ServerCore::args_of(q);
    CHECK(a1.kick_start == 0 && a1.sample_lo == 0 && a1.sample_hi == 0);
    q.tmpl.kick_start = 0;  // a plain range stays in every generation
    CHECK(ServerCore::args_of(q).sample_lo == 8);
  }

  // admission in arrival order under the budget; a failed launch advances nothing
  {
    ServerCore s;
    const uint64_t one = ServerCore::footprint(tmpl(10, 100, 4, 3));
    s.budget = one + one / 2;
    const uint64_t a = s.add(ServerCore::make(problem(3), tmpl(10, 100, 4, 3), 2));
    const uint64_t b = s.add(ServerCore::make(problem(4), tmpl(10, 100, 4, 4), 1));
    const uint64_t c = s.add(ServerCore::make(problem(5), tmpl(1, 8, 4, 5), 1));
    int calls = 0;
    auto fail = [&](const std::vector<ServerCore::Launch> &) { return ++calls, 7; };
    uint32_t res = 9, fin = 9;
    CHECK(s.tick(fail, &res, &fin) == 7 && res == 1 && fin == 0 && calls == 1);
    CHECK(s.find(a)->gen == 0 && s.ticks == 0 && s.updates == 0);
    // c would fit beside a, but b is ahead of it
    CHECK(s.find(b)->state == GLP_REQ_QUEUED && s.find(c)->state == GLP_REQ_QUEUED);
    std::vector<std::vector<uint32_t>> seen;
    auto run = [&](const std::vector<ServerCore::Launch> &ls) {
      std::vector<uint32_t> gens;
      for (const auto &l : ls)
        for (const auto &x : l.args)
          gens.push_back(x.generation);
      seen.push_back(gens);
      return 0;
    };
    CHECK(s.tick(run, &res, &fin) == 0 && res == 1 && fin == 0);
    CHECK(s.tick(run, &res, &fin) == 0 && res == 1 && fin == 1);  // a done
    CHECK(s.find(a)->state == GLP_REQ_DONE && s.find(a)->gen == 2 && s.used == 0);
    CHECK(s.tick(run, &res, &fin) == 0 && res == 2 && fin == 2);  // b and c together
    CHECK(seen.size() == 3 && seen[0] == std::vector<uint32_t>({0}) &&
          seen[1] == std::vector<uint32_t>({1}) && seen[2] == std::vector<uint32_t>({0, 0}));
    CHECK(s.ticks == 3 && s.used == 0 && s.active.empty() && s.queue.empty());
    CHECK(s.updates == 2ull * 10 * 5 * 100 + 10ull * 5 * 100 + 1ull * 5 * 8);
    // release
    CHECK(s.release(999) == 1 && s.release(a) == 0 && s.find(a) == nullptr);
    CHECK(s.release(a) == 1);
    const uint64_t d = s.add(ServerCore::make(problem(6), tmpl(1, 8, 4, 6), 3));
    CHECK(s.release(d) == 2 && s.find(d)->state == GLP_REQ_QUEUED);
  }

  // launch grouping: one launch per emission source, or per request (plain)
  {
    ServerCore s;
    s.budget = ~0ull;
    s.add(ServerCore::make(problem(7), tmpl(3, 64, 2, 7), 3));
    s.add(ServerCore::make(problem(8), tmpl(3, 64, 2, 8, 0, GLP_GEN_VQ), 3));
    s.add(ServerCore::make(problem(9), tmpl(3, 64, 2, 9), 3));
    s.admit();
    std::vector<ServerCore::Launch> ls = s.launches();
    CHECK(ls.size() == 2);
    CHECK(ls[0].problems == std::vector<void *>({problem(7), problem(9)}));
    CHECK(ls[1].problems == std::vector<void *>({problem(8)}));
    CHECK(ls[1].args[0].seed == 108 && (ls[1].args[0].flags & GLP_GEN_VQ));
    s.plain = true;
    ls = s.launches();
    CHECK(ls.size() == 3 && ls[1].problems[0] == problem(8) && ls[2].args.size() == 1);
    // requests at different generations share a launch
    auto ok = [](const std::vector<ServerCore::Launch> &) { return 0; };
    s.plain = false;
    s.tick(ok, nullptr, nullptr);
    s.add(ServerCore::make(problem(10), tmpl(3, 64, 2, 10), 1));
    s.admit();
    ls = s.launches();
    CHECK(ls[0].args.size() == 3 && ls[0].args[0].generation == 1 &&
          ls[0].args[2].generation == 0 && ls[0].args[0].haps == &bufs[7][1]);
  }

  if (failures == 0)
    std::printf("ok\n");
  return failures ? 1 : 0;
}
