// pps::gpu::GpuPostflopSolver (include/pps/gpu_cfr.h): the reference's C++
// class surface (cuda/gpu_cfr.h:141-264) as a thin wrapper over the C ABI.
// Every failing call throws std::runtime_error with the ABI's message, as
// the reference's class does for API misuse.
#include "gpu_cfr.h"

#include <cstring>
#include <memory>
#include <stdexcept>

#include "pps_gb.h"

namespace pps {
namespace gpu {

struct GpuPostflopSolver::Impl {
  pps_gb_solver* h = nullptr;
};

namespace {

void check(int rc) {
  if (rc != PPS_GB_OK) throw std::runtime_error(pps_gb_last_error());
}

pps_gb_bet_config toAbi(const pf::BetConfig& c) {
  pps_gb_bet_config o;
  std::memset(&o, 0, sizeof(o));
  if (c.betFracs.size() > PPS_GB_MAX_SIZES || c.raiseMults.size() > PPS_GB_MAX_SIZES)
    throw std::runtime_error("too many bet or raise sizes");
  o.n_bet_fracs = (int)c.betFracs.size();
  std::copy(c.betFracs.begin(), c.betFracs.end(), o.bet_fracs);
  o.n_raise_mults = (int)c.raiseMults.size();
  std::copy(c.raiseMults.begin(), c.raiseMults.end(), o.raise_mults);
  o.bet_allin = c.betAllIn;
  o.bet_geometric = c.betGeometric;
  o.max_raises = c.maxRaises;
  o.add_allin_threshold = c.addAllinThreshold;
  o.force_allin_threshold = c.forceAllinThreshold;
  o.merging_threshold = c.mergingThreshold;
  return o;
}

std::unique_ptr<pps_gb_spot> toAbi(const PostflopSpot& s) {
  std::unique_ptr<pps_gb_spot> o(new pps_gb_spot());
  std::memset(o.get(), 0, sizeof(pps_gb_spot));
  for (int i = 0; i < 5; ++i) o->board[i] = s.board[i];
  o->n_board = s.nBoard;
  std::memcpy(o->oop, s.oop.w, sizeof(o->oop));
  std::memcpy(o->ip, s.ip.w, sizeof(o->ip));
  o->pot = s.pot;
  o->stack = s.stack;
  return o;
}

ActionLabel fromAbi(const pps_gb_action& a) {
  return {(pf::ActionKind)a.kind, a.amount};
}

}  // namespace

GpuPostflopSolver::GpuPostflopSolver(const PostflopSpot& spot, const pf::BetConfig& cfg)
    : impl_(new Impl()) {
  const auto s = toAbi(spot);
  const pps_gb_bet_config c = toAbi(cfg);
  try {
    check(pps_gb_create(s.get(), &c, &impl_->h));
  } catch (...) {
    delete impl_;
    impl_ = nullptr;
    throw;
  }
  refresh();
}

GpuPostflopSolver::GpuPostflopSolver(const PostflopSpot& spot, const StreetBetConfigs& cfgs)
    : impl_(new Impl()) {
  const auto s = toAbi(spot);
  const pps_gb_bet_config c[3] = {toAbi(cfgs.street[0]), toAbi(cfgs.street[1]),
                                  toAbi(cfgs.street[2])};
  try {
    check(pps_gb_create_streets(s.get(), c, &impl_->h));
  } catch (...) {
    delete impl_;
    impl_ = nullptr;
    throw;
  }
  refresh();
}

GpuPostflopSolver::GpuPostflopSolver(const std::string& solutionPath) : impl_(new Impl()) {
  try {
    check(pps_gb_load(solutionPath.c_str(), &impl_->h));
  } catch (...) {
    delete impl_;
    impl_ = nullptr;
    throw;
  }
  refresh();
}

GpuPostflopSolver::~GpuPostflopSolver() {
  if (impl_) {
    pps_gb_destroy(impl_->h);
    delete impl_;
  }
}

void* GpuPostflopSolver::handle() const { return impl_ ? impl_->h : nullptr; }

void GpuPostflopSolver::refresh() {
  pps_gb_info info;
  check(pps_gb_get_info(impl_->h, &info));
  numNodes_ = info.num_nodes;
  maxDepth_ = info.max_depth;
  iterationsRun_ = info.iterations_run;
  totalIters_ = info.total_iterations;
}

void GpuPostflopSolver::solve(int iterations, const std::string& algo, double target) {
  const int rc = pps_gb_solve(impl_->h, iterations, algo.c_str(), target);
  refresh();
  check(rc);
}

void GpuPostflopSolver::continueSolve(int iterations, double target) {
  const int rc = pps_gb_continue(impl_->h, iterations, target);
  refresh();
  check(rc);
}

void GpuPostflopSolver::reset() {
  const int rc = pps_gb_reset(impl_->h);
  refresh();
  check(rc);
}

pf::NodeStats GpuPostflopSolver::stats() {
  pps_gb_node_stats st;
  check(pps_gb_stats(impl_->h, &st));
  pf::NodeStats o;
  o.ev0 = st.ev0;
  o.ev1 = st.ev1;
  o.expl = st.expl;
  o.pairMass = st.pair_mass;
  return o;
}

std::vector<double> GpuPostflopSolver::rootStrategy() {
  double f[PPS_GB_MAX_ACTIONS];
  int n = 0;
  check(pps_gb_root_strategy(impl_->h, f, &n));
  return std::vector<double>(f, f + n);
}

std::vector<double> GpuPostflopSolver::nodeStrategy(int decideIdx) {
  double f[PPS_GB_MAX_ACTIONS];
  int n = 0;
  check(pps_gb_node_strategy(impl_->h, decideIdx, f, &n));
  return std::vector<double>(f, f + n);
}

int GpuPostflopSolver::numDecideNodes() const {
  pps_gb_info info;
  check(pps_gb_get_info(impl_->h, &info));
  return info.num_decide_nodes;
}

DecideNodeInfo GpuPostflopSolver::decideNode(int decideIdx) const {
  pps_gb_decide_info d;
  check(pps_gb_decide_node(impl_->h, decideIdx, &d));
  DecideNodeInfo o;
  o.nodeId = d.node_id;
  o.player = d.player;
  o.depth = d.depth;
  o.nBoard = d.n_board;
  o.nCombos = d.n_combos;
  for (int a = 0; a < d.n_actions; ++a) {
    o.actions.push_back(fromAbi(d.actions[a]));
    o.children.push_back(d.children[a]);
  }
  return o;
}

ComboStrategy GpuPostflopSolver::comboStrategy(int decideIdx) {
  int na = 0, nc = 0;
  pps_gb_action acts[PPS_GB_MAX_ACTIONS];
  std::vector<int> combos(PPS_GB_COMBOS);
  std::vector<double> freqs((size_t)PPS_GB_MAX_ACTIONS * PPS_GB_COMBOS);
  check(pps_gb_combo_strategy(impl_->h, decideIdx, &na, &nc, acts, combos.data(),
                              freqs.data()));
  ComboStrategy o;
  for (int a = 0; a < na; ++a) o.actions.push_back(fromAbi(acts[a]));
  o.combos.assign(combos.begin(), combos.begin() + nc);
  o.freqs.assign(freqs.begin(), freqs.begin() + (size_t)na * nc);
  return o;
}

ComboEv GpuPostflopSolver::rootEvPerCombo() {
  ComboEv o;
  for (int p = 0; p < 2; ++p) {
    int n = 0;
    std::vector<int> combos(PPS_GB_COMBOS);
    std::vector<double> ev(PPS_GB_COMBOS), mass(PPS_GB_COMBOS);
    check(pps_gb_root_ev(impl_->h, p, &n, combos.data(), ev.data(), mass.data()));
    o.combos[p].assign(combos.begin(), combos.begin() + n);
    o.ev[p].assign(ev.begin(), ev.begin() + n);
    o.mass[p].assign(mass.begin(), mass.begin() + n);
  }
  return o;
}

NodeEv GpuPostflopSolver::nodeEv(int decideIdx) {
  int decider = 0, na = 0, nc[2] = {0, 0};
  pps_gb_action acts[PPS_GB_MAX_ACTIONS];
  std::vector<int> combos(2 * PPS_GB_COMBOS);
  std::vector<double> ev(2 * PPS_GB_COMBOS), mass(2 * PPS_GB_COMBOS),
      aev((size_t)PPS_GB_MAX_ACTIONS * PPS_GB_COMBOS);
  double agg[2], aagg[PPS_GB_MAX_ACTIONS];
  check(pps_gb_node_ev(impl_->h, decideIdx, &decider, &na, acts, nc, combos.data(), ev.data(),
                       mass.data(), agg, aev.data(), aagg));
  NodeEv o;
  o.decider = decider;
  for (int a = 0; a < na; ++a) {
    o.actions.push_back(fromAbi(acts[a]));
    NodeEv::ActionEv e;
    e.aggEv = aagg[a];
    e.perCombo.assign(aev.begin() + (size_t)a * PPS_GB_COMBOS,
                      aev.begin() + (size_t)a * PPS_GB_COMBOS + nc[decider]);
    o.actionEv.push_back(e);
  }
  for (int p = 0; p < 2; ++p) {
    const size_t b = (size_t)p * PPS_GB_COMBOS;
    o.side[p].combos.assign(combos.begin() + b, combos.begin() + b + nc[p]);
    o.side[p].ev.assign(ev.begin() + b, ev.begin() + b + nc[p]);
    o.side[p].mass.assign(mass.begin() + b, mass.begin() + b + nc[p]);
    o.side[p].aggEv = agg[p];
  }
  return o;
}

RunoutSummary GpuPostflopSolver::runoutSummary(int decideIdx, int actionIdx) {
  int decider = 0, na = 0, nb = 0;
  pps_gb_action acts[PPS_GB_MAX_ACTIONS];
  int cards[52], next[52], nf[52];
  std::vector<double> freq(52 * PPS_GB_MAX_ACTIONS), agg(104);
  check(pps_gb_runout_summary(impl_->h, decideIdx, actionIdx, &decider, &na, acts, &nb, cards,
                              next, nf, freq.data(), agg.data()));
  RunoutSummary o;
  o.decider = decider;
  for (int a = 0; a < na; ++a) o.actions.push_back(fromAbi(acts[a]));
  for (int b = 0; b < nb; ++b) {
    RunoutSummary::Branch br;
    br.card = cards[b];
    br.nextDecide = next[b];
    br.freq.assign(freq.begin() + b * PPS_GB_MAX_ACTIONS,
                   freq.begin() + b * PPS_GB_MAX_ACTIONS + nf[b]);
    br.aggEv[0] = agg[2 * b];
    br.aggEv[1] = agg[2 * b + 1];
    o.branches.push_back(br);
  }
  return o;
}

std::vector<uint8_t> GpuPostflopSolver::playerCards(int player) const {
  std::vector<uint8_t> c(2 * PPS_GB_COMBOS);
  int n = 0;
  check(pps_gb_player_cards(impl_->h, player, c.data(), &n));
  c.resize(2 * n);
  return c;
}

int GpuPostflopSolver::numBaseCombos(int player) const {
  return (int)playerCards(player).size() / 2;
}

std::vector<double> GpuPostflopSolver::playerWeights(int player) const {
  std::vector<double> w(PPS_GB_COMBOS);
  int n = 0;
  check(pps_gb_player_weights(impl_->h, player, w.data(), &n));
  w.resize(n);
  return w;
}

TreeStructure GpuPostflopSolver::treeStructure() const {
  int nn = 0, nc = 0;
  check(pps_gb_tree_structure(impl_->h, nullptr, nullptr, nullptr, nullptr, &nn, &nc));
  TreeStructure t;
  t.kinds.resize(nn);
  t.childBase.resize(nn);
  t.children.resize(nc);
  t.boards.resize((size_t)nn * 5);
  check(pps_gb_tree_structure(impl_->h, t.kinds.data(), t.childBase.data(), t.children.data(),
                              t.boards.data(), &nn, &nc));
  return t;
}

void GpuPostflopSolver::saveCompressed(const std::string& path) const {
  check(pps_gb_save_compressed(impl_->h, path.c_str()));
}

void GpuPostflopSolver::save(const std::string& path) const {
  check(pps_gb_save(impl_->h, path.c_str()));
}

void GpuPostflopSolver::debugDump() { check(pps_gb_debug_dump(impl_->h)); }

}  // namespace gpu
}  // namespace pps
