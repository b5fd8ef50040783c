// The C ABI (include/pps_gb.h) over SolverCore. Every entry point catches
// everything, stores the message in a thread-local string and returns a
// status code; nothing here exits the process.
#include "pps_gb.h"

#include <algorithm>
#include <cstring>
#include <new>
#include <string>

#include "batch.h"
#include "compiler.h"
#include "engine.h"
#include "forest.h"
#include "noalloc.h"
#include "solver.h"

using pps::gb::Error;
using pps::gb::SolverCore;

struct pps_gb_solver {
  std::unique_ptr<SolverCore> core;
};

struct pps_gb_batch {
  std::unique_ptr<pps::gb::BatchServer> server;
};

namespace {

thread_local std::string g_lastError;

int fail(int code, const std::string& msg) {
  g_lastError = msg;
  return code;
}

template <typename F>
int guarded(F&& f) {
  try {
    f();
    return PPS_GB_OK;
  } catch (const Error& e) {
    return fail(e.code, e.msg);
  } catch (const std::bad_alloc&) {
    return fail(PPS_GB_E_MEMORY, "host allocation failed");
  } catch (const std::exception& e) {
    return fail(PPS_GB_E_ARG, e.what());
  } catch (...) {
    return fail(PPS_GB_E_ARG, "unknown error");
  }
}

pps::pf::BetConfig toConfig(const pps_gb_bet_config& c) {
  if (c.n_bet_fracs < 0 || c.n_bet_fracs > PPS_GB_MAX_SIZES || c.n_raise_mults < 0 ||
      c.n_raise_mults > PPS_GB_MAX_SIZES)
    throw Error{PPS_GB_E_ARG, "bad bet/raise size count"};
  pps::pf::BetConfig o;
  o.betFracs.assign(c.bet_fracs, c.bet_fracs + c.n_bet_fracs);
  o.raiseMults.assign(c.raise_mults, c.raise_mults + c.n_raise_mults);
  o.betAllIn = c.bet_allin != 0;
  o.betGeometric = c.bet_geometric != 0;
  o.maxRaises = c.max_raises;
  o.addAllinThreshold = c.add_allin_threshold;
  o.forceAllinThreshold = c.force_allin_threshold;
  o.mergingThreshold = c.merging_threshold;
  return o;
}

pps::gpu::PostflopSpot toSpot(const pps_gb_spot& s) {
  pps::gpu::PostflopSpot o;
  if (s.n_board < 3 || s.n_board > 5)
    throw Error{PPS_GB_E_ARG, "board must be 3, 4 or 5 cards"};
  o.nBoard = s.n_board;
  for (int i = 0; i < 5; ++i) o.board[i] = i < s.n_board ? s.board[i] : 0;
  std::memcpy(o.oop.w, s.oop, sizeof(o.oop.w));
  std::memcpy(o.ip.w, s.ip, sizeof(o.ip.w));
  o.pot = s.pot;
  o.stack = s.stack;
  return o;
}

pps_gb_action toAction(const pps::gpu::ActionLabel& a) {
  pps_gb_action o;
  o.kind = (int32_t)a.kind;
  o.amount = a.amount;
  return o;
}

pps::gpu::StreetBetConfigs toConfigs(const pps_gb_bet_config* cfgs, int n) {
  if (!cfgs || (n != 1 && n != 3)) throw Error{PPS_GB_E_ARG, "cfgs must hold 1 or 3 configs"};
  pps::gpu::StreetBetConfigs c;
  for (int k = 0; k < 3; ++k) c.street[k] = toConfig(cfgs[n == 3 ? k : 0]);
  return c;
}

pps::gb::BatchServer& server(pps_gb_batch* b) {
  if (!b || !b->server) throw Error{PPS_GB_E_ARG, "null batch handle"};
  return *b->server;
}

void toResult(const pps::gb::BatchResult& r, pps_gb_batch_result* o) {
  std::memset(o, 0, sizeof(*o));
  o->ticket = r.ticket;
  o->status = r.status;
  o->converged = r.converged ? 1 : 0;
  o->iterations = r.iterations;
  o->num_nodes = r.numNodes;
  o->ev0 = r.ev0;
  o->ev1 = r.ev1;
  o->exploitability = r.expl;
  o->target = r.target;
  o->pair_mass = r.pairMass;
  o->submit_ms = r.submitMs;
  o->admit_ms = r.admitMs;
  o->finish_ms = r.finishMs;
  o->device_bytes = (int64_t)r.deviceBytes;
  o->root_actions = (int32_t)r.rootActions.size();
  o->root_combos = r.rootCombos;
  for (size_t a = 0; a < r.rootActions.size() && a < PPS_GB_MAX_ACTIONS; ++a) {
    o->root_action[a].kind = (int32_t)r.rootActions[a].kind;
    o->root_action[a].amount = r.rootActions[a].amount;
    o->root_freqs[a] = a < r.rootFreqs.size() ? r.rootFreqs[a] : 0.0;
  }
  std::strncpy(o->error, r.error.c_str(), sizeof(o->error) - 1);
}

SolverCore& core(pps_gb_solver* h) {
  if (!h || !h->core) throw Error{PPS_GB_E_ARG, "null solver handle"};
  return *h->core;
}

}  // namespace

extern "C" {

const char* pps_gb_last_error(void) { return g_lastError.c_str(); }

int pps_gb_abi_version(void) { return PPS_GB_ABI_VERSION; }

void pps_gb_bet_config_default(pps_gb_bet_config* cfg) {
  if (!cfg) return;
  std::memset(cfg, 0, sizeof(*cfg));
  const pps::pf::BetConfig d;
  cfg->n_bet_fracs = (int)d.betFracs.size();
  std::copy(d.betFracs.begin(), d.betFracs.end(), cfg->bet_fracs);
  cfg->n_raise_mults = (int)d.raiseMults.size();
  std::copy(d.raiseMults.begin(), d.raiseMults.end(), cfg->raise_mults);
  cfg->bet_allin = d.betAllIn;
  cfg->bet_geometric = d.betGeometric;
  cfg->max_raises = d.maxRaises;
  cfg->add_allin_threshold = d.addAllinThreshold;
  cfg->force_allin_threshold = d.forceAllinThreshold;
  cfg->merging_threshold = d.mergingThreshold;
}

int pps_gb_create(const pps_gb_spot* spot, const pps_gb_bet_config* cfg,
                  pps_gb_solver** out) {
  return guarded([&] {
    if (!spot || !cfg || !out) throw Error{PPS_GB_E_ARG, "null argument"};
    *out = nullptr;
    pps::gpu::StreetBetConfigs c;
    c.street[0] = c.street[1] = c.street[2] = toConfig(*cfg);
    auto* h = new pps_gb_solver();
    try {
      h->core.reset(new SolverCore(toSpot(*spot), c, false));
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}

int pps_gb_create_streets(const pps_gb_spot* spot, const pps_gb_bet_config cfgs[3],
                          pps_gb_solver** out) {
  return guarded([&] {
    if (!spot || !cfgs || !out) throw Error{PPS_GB_E_ARG, "null argument"};
    *out = nullptr;
    pps::gpu::StreetBetConfigs c;
    for (int k = 0; k < 3; ++k) c.street[k] = toConfig(cfgs[k]);
    auto* h = new pps_gb_solver();
    try {
      h->core.reset(new SolverCore(toSpot(*spot), c, true));
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}

int pps_gb_load(const char* path, pps_gb_solver** out) {
  return guarded([&] {
    if (!path || !out) throw Error{PPS_GB_E_ARG, "null argument"};
    *out = nullptr;
    auto* h = new pps_gb_solver();
    try {
      h->core = SolverCore::load(path);
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}

void pps_gb_destroy(pps_gb_solver* h) {
  try {
    delete h;
  } catch (...) {
  }
}

int pps_gb_solve(pps_gb_solver* h, int iterations, const char* algo, double target) {
  return guarded([&] { core(h).solve(iterations, algo ? algo : "dcfr", target); });
}

int pps_gb_continue(pps_gb_solver* h, int iterations, double target) {
  return guarded([&] { core(h).continueSolve(iterations, target); });
}

int pps_gb_reset(pps_gb_solver* h) {
  return guarded([&] { core(h).reset(); });
}

int pps_gb_get_info(pps_gb_solver* h, pps_gb_info* out) {
  return guarded([&] {
    SolverCore& s = core(h);
    if (!out) throw Error{PPS_GB_E_ARG, "null argument"};
    std::memset(out, 0, sizeof(*out));
    const auto& t = s.tree();
    out->num_nodes = (int32_t)t.nodes.size();
    out->max_depth = t.maxDepth;
    out->num_decide_nodes = (int32_t)t.decideNodes.size();
    out->iterations_run = s.iterationsRun();
    out->total_iterations = s.totalIterations();
    out->n_base[0] = t.side[0].n;
    out->n_base[1] = t.side[1].n;
    out->row_total = t.rowTotal;
    out->empty = t.empty ? 1 : 0;
    if (s.engine()) {
      out->launches_per_iteration = s.engine()->launchesPerIteration();
      out->device_bytes = (int64_t)s.engine()->deviceBytes();
      out->h2d_bytes = s.engine()->h2dBytes();
      out->d2h_bytes = s.engine()->d2hBytes();
      out->engine = s.engine()->engineKind();
      out->compensated = s.engine()->compensated() ? 1 : 0;
    }
  });
}

int pps_gb_stats(pps_gb_solver* h, pps_gb_node_stats* out) {
  return guarded([&] {
    if (!out) throw Error{PPS_GB_E_ARG, "null argument"};
    const auto st = core(h).stats();
    out->ev0 = st.ev0;
    out->ev1 = st.ev1;
    out->expl = st.expl;
    out->pair_mass = st.pairMass;
  });
}

int pps_gb_root_strategy(pps_gb_solver* h, double* freq, int* n_actions) {
  return guarded([&] {
    const auto f = core(h).rootStrategy();
    *n_actions = (int)f.size();
    std::copy(f.begin(), f.end(), freq);
  });
}

int pps_gb_node_strategy(pps_gb_solver* h, int decide_idx, double* freq, int* n_actions) {
  return guarded([&] {
    const auto f = core(h).nodeStrategy(decide_idx);
    *n_actions = (int)f.size();
    std::copy(f.begin(), f.end(), freq);
  });
}

int pps_gb_decide_node(pps_gb_solver* h, int decide_idx, pps_gb_decide_info* out) {
  return guarded([&] {
    const auto d = core(h).decideNode(decide_idx);
    std::memset(out, 0, sizeof(*out));
    out->node_id = d.nodeId;
    out->player = d.player;
    out->depth = d.depth;
    out->n_board = d.nBoard;
    out->n_combos = d.nCombos;
    out->n_actions = (int)d.actions.size();
    for (size_t a = 0; a < d.actions.size(); ++a) {
      out->actions[a] = toAction(d.actions[a]);
      out->children[a] = d.children[a];
    }
  });
}

int pps_gb_combo_strategy(pps_gb_solver* h, int decide_idx, int* n_actions, int* n_combos,
                          pps_gb_action* actions, int* combos, double* freqs) {
  return guarded([&] {
    const auto cs = core(h).comboStrategy(decide_idx);
    *n_actions = (int)cs.actions.size();
    *n_combos = (int)cs.combos.size();
    for (size_t a = 0; a < cs.actions.size(); ++a) actions[a] = toAction(cs.actions[a]);
    std::copy(cs.combos.begin(), cs.combos.end(), combos);
    std::copy(cs.freqs.begin(), cs.freqs.end(), freqs);
  });
}

int pps_gb_root_ev(pps_gb_solver* h, int player, int* n, int* combos, double* ev,
                   double* mass) {
  return guarded([&] {
    if (player < 0 || player > 1)
      throw Error{PPS_GB_E_INDEX, "player must be 0 (OOP) or 1 (IP)"};
    const auto r = core(h).rootEvPerCombo();
    *n = (int)r.combos[player].size();
    std::copy(r.combos[player].begin(), r.combos[player].end(), combos);
    std::copy(r.ev[player].begin(), r.ev[player].end(), ev);
    std::copy(r.mass[player].begin(), r.mass[player].end(), mass);
  });
}

int pps_gb_node_ev(pps_gb_solver* h, int decide_idx, int* decider, int* n_actions,
                   pps_gb_action* actions, int* n_combos, int* combos, double* ev,
                   double* mass, double* agg_ev, double* action_ev, double* action_agg) {
  return guarded([&] {
    const auto r = core(h).nodeEv(decide_idx);
    *decider = r.decider;
    *n_actions = (int)r.actions.size();
    for (size_t a = 0; a < r.actions.size(); ++a) {
      actions[a] = toAction(r.actions[a]);
      action_agg[a] = r.actionEv[a].aggEv;
      std::copy(r.actionEv[a].perCombo.begin(), r.actionEv[a].perCombo.end(),
                action_ev + a * PPS_GB_COMBOS);
    }
    for (int p = 0; p < 2; ++p) {
      const auto& S = r.side[p];
      n_combos[p] = (int)S.combos.size();
      std::copy(S.combos.begin(), S.combos.end(), combos + p * PPS_GB_COMBOS);
      std::copy(S.ev.begin(), S.ev.end(), ev + p * PPS_GB_COMBOS);
      std::copy(S.mass.begin(), S.mass.end(), mass + p * PPS_GB_COMBOS);
      agg_ev[p] = S.aggEv;
    }
  });
}

int pps_gb_runout_summary(pps_gb_solver* h, int decide_idx, int action_idx, int* decider,
                          int* n_actions, pps_gb_action* actions, int* n_branches,
                          int* cards, int* next_decide, int* n_freq, double* freq,
                          double* agg_ev) {
  return guarded([&] {
    const auto r = core(h).runoutSummary(decide_idx, action_idx);
    *decider = r.decider;
    *n_actions = (int)r.actions.size();
    for (size_t a = 0; a < r.actions.size(); ++a) actions[a] = toAction(r.actions[a]);
    *n_branches = (int)r.branches.size();
    for (size_t b = 0; b < r.branches.size(); ++b) {
      const auto& br = r.branches[b];
      cards[b] = br.card;
      next_decide[b] = br.nextDecide;
      n_freq[b] = (int)br.freq.size();
      std::copy(br.freq.begin(), br.freq.end(), freq + b * PPS_GB_MAX_ACTIONS);
      agg_ev[2 * b] = br.aggEv[0];
      agg_ev[2 * b + 1] = br.aggEv[1];
    }
  });
}

int pps_gb_player_cards(pps_gb_solver* h, int player, uint8_t* cards, int* n) {
  return guarded([&] {
    const auto c = core(h).playerCards(player);
    *n = (int)c.size() / 2;
    std::copy(c.begin(), c.end(), cards);
  });
}

int pps_gb_player_weights(pps_gb_solver* h, int player, double* w, int* n) {
  return guarded([&] {
    const auto v = core(h).playerWeights(player);
    *n = (int)v.size();
    std::copy(v.begin(), v.end(), w);
  });
}

int pps_gb_tree_structure(pps_gb_solver* h, uint8_t* kinds, int* child_base, int* children,
                          uint8_t* boards, int* n_nodes, int* n_children) {
  return guarded([&] {
    const auto& t = core(h).tree();
    *n_nodes = (int)t.nodes.size();
    *n_children = (int)t.children.size();
    if (!kinds) return;
    const auto s = core(h).treeStructure();
    std::copy(s.kinds.begin(), s.kinds.end(), kinds);
    std::copy(s.childBase.begin(), s.childBase.end(), child_base);
    std::copy(s.children.begin(), s.children.end(), children);
    std::copy(s.boards.begin(), s.boards.end(), boards);
  });
}

int pps_gb_save(pps_gb_solver* h, const char* path) {
  return guarded([&] {
    if (!path) throw Error{PPS_GB_E_ARG, "null path"};
    core(h).save(path);
  });
}

int pps_gb_save_compressed(pps_gb_solver* h, const char* path) {
  return guarded([&] {
    if (!path) throw Error{PPS_GB_E_ARG, "null path"};
    core(h).save(path, true);
  });
}

int pps_gb_debug_dump(pps_gb_solver* h) {
  return guarded([&] { core(h).debugDump(); });
}

int pps_gb_read_rows(pps_gb_solver* h, int which, float* out, int64_t cap, int64_t* n) {
  return guarded([&] {
    SolverCore& s = core(h);
    if (which != 0 && which != 1) throw Error{PPS_GB_E_ARG, "which must be 0 or 1"};
    *n = s.tree().rowTotal;
    if (!out || !s.engine()) return;
    if (cap < s.tree().rowTotal) throw Error{PPS_GB_E_ARG, "row buffer too small"};
    const auto rows = s.engine()->denseRows(which);
    std::copy(rows.begin(), rows.end(), out);
  });
}

int pps_gb_write_rows(pps_gb_solver* h, int which, const float* in, int64_t n) {
  return guarded([&] {
    SolverCore& s = core(h);
    if (which != 0 && which != 1) throw Error{PPS_GB_E_ARG, "which must be 0 or 1"};
    if (!s.engine()) throw Error{PPS_GB_E_STATE, "solver compiled to empty ranges"};
    s.engine()->setDenseRows(which, std::vector<float>(in, in + n));
  });
}

int pps_gb_walk(pps_gb_solver* h, int traverser, int mode, double* root_cfv, double* value) {
  return guarded([&] {
    if (traverser < 0 || traverser > 1) throw Error{PPS_GB_E_INDEX, "bad traverser"};
    if (mode != 0 && mode != 1) throw Error{PPS_GB_E_ARG, "mode must be 0 (EV) or 1 (BR)"};
    std::vector<double> row;
    *value = core(h).walkValue(traverser, mode == 0 ? pps::gb::kModeEV : pps::gb::kModeBR,
                               &row);
    if (root_cfv) std::copy(row.begin(), row.end(), root_cfv);
  });
}

int pps_gb_set_engine(pps_gb_solver* h, int engine) {
  return guarded([&] {
    SolverCore& s = core(h);
    if (s.engine()) s.engine()->setEngineKind(engine);
  });
}

int pps_gb_set_launch_shape(pps_gb_solver* h, const pps_gb_launch_shape* shape) {
  return guarded([&] {
    SolverCore& s = core(h);
    if (!shape) throw Error{PPS_GB_E_ARG, "null argument"};
    pps::gb::LaunchShape ls;
    ls.plan = shape->plan;
    ls.fwdCap = shape->fwd_cap;
    ls.bwdCap = shape->bwd_cap;
    ls.sdCap = shape->sd_cap;
    ls.fdCap = shape->fd_cap;
    if (s.engine()) s.engine()->setShape(ls);
  });
}

int pps_gb_get_launch_shape(pps_gb_solver* h, pps_gb_launch_shape* out) {
  return guarded([&] {
    SolverCore& s = core(h);
    if (!out) throw Error{PPS_GB_E_ARG, "null argument"};
    std::memset(out, 0, sizeof(*out));
    if (!s.engine()) return;
    const pps::gb::LaunchShape ls = s.engine()->shape();
    out->plan = ls.plan;
    out->fwd_cap = ls.fwdCap;
    out->bwd_cap = ls.bwdCap;
    out->sd_cap = ls.sdCap;
    out->fd_cap = ls.fdCap;
  });
}

int pps_gb_set_compensated(pps_gb_solver* h, int on) {
  return guarded([&] {
    SolverCore& s = core(h);
    if (s.engine()) s.engine()->setCompensated(on != 0);
  });
}

int pps_gb_time_iterations(pps_gb_solver* h, int n, double* ms) {
  return guarded([&] {
    if (!ms || n < 0) throw Error{PPS_GB_E_ARG, "bad arguments"};
    *ms = core(h).timeIterations(n);
  });
}

int pps_gb_probe_bounded_wait(pps_gb_solver* h, int spins) {
  return guarded([&] {
    // At most the records' own bound (65,536 polls a round), so that the
    // probe ends as quickly as their give-up path does.
    if (spins < 1 || spins > (1 << 16)) throw Error{PPS_GB_E_ARG, "spins must be in [1, 65536]"};
    core(h).probeBoundedWait(spins);
  });
}

int pps_gb_profile(pps_gb_solver* h, int n, int flags, pps_gb_kernel_stat* out, int cap,
                   int* n_out) {
  return guarded([&] {
    if (!out || !n_out || n < 1) throw Error{PPS_GB_E_ARG, "bad arguments"};
    const auto stats = core(h).profile(n, (flags & 1) != 0);
    *n_out = std::min<int>((int)stats.size(), cap);
    for (int i = 0; i < *n_out; ++i) {
      std::memset(out[i].name, 0, sizeof(out[i].name));
      std::strncpy(out[i].name, stats[i].name.c_str(), sizeof(out[i].name) - 1);
      out[i].launches = stats[i].launches;
      out[i].ms = stats[i].ms;
      out[i].algo_bytes = stats[i].bytes;
    }
  });
}

int pps_gb_solve_noalloc(const pps_gb_spot* spot, const pps_gb_bet_config* cfg,
                         float* d_regret, float* d_strat, int64_t row_capacity,
                         int first_iteration, int iterations, void* stream, int64_t* n_rows) {
  return guarded([&] {
    if (!spot || !cfg) throw Error{PPS_GB_E_ARG, "null argument"};
    pps::gb::noallocSolve(toSpot(*spot), toConfig(*cfg), d_regret, d_strat, row_capacity,
                          first_iteration, iterations, static_cast<cudaStream_t>(stream),
                          n_rows);
  });
}

void pps_gb_batch_config_default(pps_gb_batch_config* cfg) {
  if (!cfg) return;
  std::memset(cfg, 0, sizeof(*cfg));
  const pps::gb::BatchConfig d;
  cfg->hbm_budget = d.budget;
  cfg->check_every = d.checkEvery;
  cfg->fixed_checks = d.fixedChecks ? 1 : 0;
  cfg->max_iterations = d.maxIterations;
  cfg->compile_threads = d.threads;
  std::strncpy(cfg->algo, d.algo.c_str(), sizeof(cfg->algo) - 1);
}

int pps_gb_batch_create(const pps_gb_batch_config* cfg, pps_gb_batch** out) {
  return guarded([&] {
    if (!out) throw Error{PPS_GB_E_ARG, "null argument"};
    *out = nullptr;
    pps::gb::BatchConfig c;
    if (cfg) {
      c.budget = cfg->hbm_budget;
      c.checkEvery = cfg->check_every;
      c.fixedChecks = cfg->fixed_checks != 0;
      c.maxIterations = cfg->max_iterations;
      c.threads = cfg->compile_threads;
      const size_t n = strnlen(cfg->algo, sizeof(cfg->algo));
      if (n) c.algo.assign(cfg->algo, n);
    }
    auto* b = new pps_gb_batch();
    try {
      b->server.reset(new pps::gb::BatchServer(c));
    } catch (...) {
      delete b;
      throw;
    }
    *out = b;
  });
}

void pps_gb_batch_destroy(pps_gb_batch* b) { delete b; }

int pps_gb_batch_set_budget(pps_gb_batch* b, int64_t bytes) {
  return guarded([&] { server(b).setBudget(bytes); });
}

int pps_gb_batch_submit(pps_gb_batch* b, const pps_gb_spot* spot, const pps_gb_bet_config* cfgs,
                        int n_cfgs, double target, int64_t* ticket) {
  return guarded([&] {
    if (!spot || !ticket) throw Error{PPS_GB_E_ARG, "null argument"};
    *ticket = server(b).submit(toSpot(*spot), toConfigs(cfgs, n_cfgs), n_cfgs == 3, target);
  });
}

int pps_gb_batch_run(pps_gb_batch* b, double timeout_s) {
  bool all = false;
  const int rc = guarded([&] { all = server(b).run(timeout_s); });
  return rc != PPS_GB_OK ? rc : all ? PPS_GB_OK : PPS_GB_PENDING;
}

int pps_gb_batch_start(pps_gb_batch* b) { return guarded([&] { server(b).start(); }); }
int pps_gb_batch_stop(pps_gb_batch* b) { return guarded([&] { server(b).stop(); }); }

int pps_gb_batch_poll(pps_gb_batch* b, int64_t ticket, pps_gb_batch_result* out) {
  bool done = false;
  const int rc = guarded([&] {
    pps::gb::BatchResult r;
    done = server(b).poll(ticket, &r);
    if (done && out) toResult(r, out);
  });
  return rc != PPS_GB_OK ? rc : done ? PPS_GB_OK : PPS_GB_PENDING;
}

int pps_gb_batch_wait(pps_gb_batch* b, int64_t ticket, double timeout_s,
                      pps_gb_batch_result* out) {
  bool done = false;
  const int rc = guarded([&] {
    pps::gb::BatchResult r;
    done = server(b).wait(ticket, timeout_s, &r);
    if (done && out) toResult(r, out);
  });
  return rc != PPS_GB_OK ? rc : done ? PPS_GB_OK : PPS_GB_PENDING;
}

int pps_gb_batch_collect(pps_gb_batch* b, pps_gb_batch_result* out, int cap, int* n_out) {
  return guarded([&] {
    if (!n_out || (cap > 0 && !out)) throw Error{PPS_GB_E_ARG, "null argument"};
    const auto rs = server(b).collect(cap > 0 ? (size_t)cap : 0);
    for (size_t i = 0; i < rs.size(); ++i) toResult(rs[i], &out[i]);
    *n_out = (int)rs.size();
  });
}

int pps_gb_batch_root_rows(pps_gb_batch* b, int64_t ticket, float* out, int64_t cap,
                           int64_t* n_out) {
  return guarded([&] {
    if (!n_out) throw Error{PPS_GB_E_ARG, "null argument"};
    pps::gb::BatchResult r;
    if (!server(b).poll(ticket, &r)) throw Error{PPS_GB_E_STATE, "request not finished"};
    *n_out = (int64_t)r.rootRows.size();
    if ((int64_t)r.rootRows.size() > cap || (!out && !r.rootRows.empty()))
      throw Error{PPS_GB_E_ARG, "buffer too small: need " + std::to_string(r.rootRows.size())};
    std::copy(r.rootRows.begin(), r.rootRows.end(), out);
  });
}

int pps_gb_batch_get_info(pps_gb_batch* b, pps_gb_batch_info* out) {
  return guarded([&] {
    if (!out) throw Error{PPS_GB_E_ARG, "null argument"};
    const pps::gb::BatchInfo i = server(b).info();
    out->submitted = i.submitted;
    out->compiling = i.compiling;
    out->waiting = i.waiting;
    out->active = i.active;
    out->done = i.done;
    out->failed = i.failed;
    out->used_bytes = i.usedBytes;
    out->device_bytes = i.deviceBytes;
    out->budget = i.budget;
    out->epochs = i.epochs;
    out->spot_iterations = i.spotIterations;
    out->captures = i.captures;
    out->peak_active = i.peakActive;
    out->peak_used_bytes = i.peakUsed;
    out->check_every = i.checkEvery;
    out->admit_ms = i.admitMs;
    out->iterate_ms = i.iterateMs;
    out->check_ms = i.checkMs;
    out->retire_ms = i.retireMs;
    out->idle_ms = i.idleMs;
    out->max_iterations = i.maxIterations;
  });
}

int pps_gb_batch_footprint(const pps_gb_spot* spot, const pps_gb_bet_config* cfgs, int n_cfgs,
                           int64_t* bytes) {
  return guarded([&] {
    if (!spot || !bytes) throw Error{PPS_GB_E_ARG, "null argument"};
    const auto cs = pps::gb::compileSpot(toSpot(*spot), toConfigs(cfgs, n_cfgs), n_cfgs == 3);
    *bytes = (int64_t)cs->bytes;
  });
}

int pps_gb_layout_digest(const pps_gb_spot* spot, const pps_gb_bet_config* cfgs, int n_cfgs,
                         uint64_t* digest) {
  return guarded([&] {
    if (!spot || !digest) throw Error{PPS_GB_E_ARG, "null argument"};
    const pps::gb::Tree t = pps::gb::compileTree(toSpot(*spot), toConfigs(cfgs, n_cfgs),
                                                 n_cfgs == 3);
    *digest = t.empty ? 0 : pps::gb::layoutDigest(pps::gb::buildLayout(t));
  });
}

int pps_gb_compile_export(const pps_gb_spot* spot, const pps_gb_bet_config* cfgs, int n_cfgs,
                          pps_gb_array_cb cb, void* user) {
  return guarded([&] {
    if (!spot || !cfgs || !cb || (n_cfgs != 1 && n_cfgs != 3))
      throw Error{PPS_GB_E_ARG, "bad export arguments"};
    pps::gpu::StreetBetConfigs c;
    for (int k = 0; k < 3; ++k) c.street[k] = toConfig(cfgs[n_cfgs == 3 ? k : 0]);
    const pps::gb::Tree t = pps::gb::compileTree(toSpot(*spot), c, n_cfgs == 3);
    pps::gb::exportReference(t, [&](const char* name, char dt, const void* d, int64_t n) {
      cb(user, name, dt, d, n);
    });
  });
}

int pps_gb_hand_keys(const uint8_t* cards, int n, uint64_t* keys) {
  return guarded([&] {
    for (int i = 0; i < n; ++i) {
      pps::Card c[7];
      for (int k = 0; k < 7; ++k) c[k] = cards[7 * i + k];
      keys[i] = pps::handKey(pps::evaluate7(c));
    }
  });
}

int pps_gb_bet_actions(int64_t pot_base, int64_t stack, const pps_gb_bet_config* cfg,
                       int64_t sc0, int64_t sc1, int actor, int after_allin, int num_bets,
                       int num_streets, pps_gb_action* out, int* n) {
  return guarded([&] {
    const auto acts = pps::pf::betActions(pot_base, stack, toConfig(*cfg), sc0, sc1, actor,
                                          after_allin != 0, num_bets, num_streets);
    if ((int)acts.size() > PPS_GB_MAX_ACTIONS) throw Error{PPS_GB_E_TOO_WIDE, "too many actions"};
    *n = (int)acts.size();
    for (size_t i = 0; i < acts.size(); ++i) {
      out[i].kind = (int32_t)acts[i].kind;
      out[i].amount = acts[i].amount;
    }
  });
}

int pps_gb_parse_range(const char* text, double* w) {
  return guarded([&] {
    if (!text || !w) throw Error{PPS_GB_E_ARG, "null argument"};
    const pps::Range r = pps::parseRange(text);
    std::copy(r.w, r.w + PPS_GB_COMBOS, w);
  });
}

}  // extern "C"
