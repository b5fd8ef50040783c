"""pps_native: the reference's Python binding surface (python/pps_native.cpp:
514-551) over the C ABI of libpps_gb.so.

    import pps
    s = pps.Solver(board="Qs9h2d", oop="TT+,AKo", ip="AQ+,KQs",
                   pot=200, stack=500, bets="0.75,a", raises="2.5,3")
    s.solve(2000)                    # or s.solve(max_iters=100000, target=0.1)
    s.stats()                        # {"ev_oop", "ev_ip", "exploitability", "pair_mass"}
    s.strategy()                     # labeled per-combo root strategy
    s.save("spot.sol"); t = pps.Solver.load("spot.sol"); t.continue_solve(500)

Same constructor keywords, methods, properties and returned dict keys as
the reference; errors raise RuntimeError like the reference binding's
translated std::runtime_error. Extension keywords: ``streets`` (per-street
bet configs, see Solver.__init__).
"""
from __future__ import annotations

import ctypes as C
from typing import Any, Dict, List, Optional, Sequence

import numpy as np

from . import _abi
from ._abi import lib, check

_RANKS = "23456789TJQKA"
_SUITS = "cdhs"
_KIND = {0: "fold", 1: "check", 2: "call", 3: "bet", 4: "raise", 5: "allin"}


def _card(text: str, i: int) -> int:
    if i + 1 >= len(text) or text[i] == ",":
        raise RuntimeError("bad card text '%s'" % text[:2])
    r = text[i].upper()
    s = text[i + 1].lower()
    if r not in _RANKS:
        raise RuntimeError("bad card rank '%s'" % text[i])
    if s not in _SUITS:
        raise RuntimeError("bad card suit '%s'" % text[i + 1])
    return _SUITS.index(s) * 13 + _RANKS.index(r)


def card_text(c: int) -> str:
    return _RANKS[c % 13] + _SUITS[c // 13]


def parse_board(board: Any) -> List[int]:
    if isinstance(board, str):
        joined = board
    elif isinstance(board, (list, tuple)):
        joined = "".join(str(c) for c in board)
    else:
        raise RuntimeError("board must be a string or a list of card strings")
    if len(joined) % 2 or not 6 <= len(joined) <= 10:
        raise RuntimeError('board must be 3, 4 or 5 cards (e.g. "Qs9h2d")')
    return [_card(joined, i) for i in range(0, len(joined), 2)]


def parse_range(text: str) -> np.ndarray:
    w = (C.c_double * _abi.COMBOS)()
    check(lib.pps_gb_parse_range(text.encode(), w))
    return np.frombuffer(w, dtype=np.float64).copy()


def _range_arg(r: Any) -> np.ndarray:
    if isinstance(r, str):
        return parse_range(r)
    if isinstance(r, dict):
        return parse_range(",".join("%s:%r" % (k, float(v)) for k, v in r.items()))
    if isinstance(r, (list, tuple, np.ndarray)):
        a = np.asarray(r, dtype=np.float64)
        if a.shape != (_abi.COMBOS,):
            raise RuntimeError("range list must have exactly 1326 weights")
        return a.copy()
    raise RuntimeError("range must be a string, dict or 1326-float list")


def _bet_config(bets: Any, raises: Any, max_raises: int) -> _abi.BetConfig:
    cfg = _abi.BetConfig()
    lib.pps_gb_bet_config_default(C.byref(cfg))
    fracs: List[float] = []
    allin = geo = False
    toks = bets.split(",") if isinstance(bets, str) else list(bets)
    for tok in toks:
        if isinstance(tok, str):
            t = tok.strip()
            if not t:
                continue
            if t in ("a", "A", "allin"):
                allin = True
            elif t in ("e", "E", "geo"):
                geo = True
            else:
                try:
                    fracs.append(float(t))
                except ValueError:
                    raise RuntimeError("bad bet size token '%s'" % t) from None
        else:
            fracs.append(float(tok))
    if isinstance(raises, str):
        mults = [float(t) for t in raises.split(",") if t.strip()]
    else:
        mults = [float(x) for x in raises]
    if not fracs and not allin and not geo:
        raise RuntimeError('empty bet abstraction: pass at least one size (e.g. "0.75,a")')
    if len(fracs) > _abi.MAX_SIZES or len(mults) > _abi.MAX_SIZES:
        raise RuntimeError("too many bet or raise sizes")
    cfg.n_bet_fracs = len(fracs)
    for i, f in enumerate(fracs):
        cfg.bet_fracs[i] = f
    cfg.n_raise_mults = len(mults)
    for i, m in enumerate(mults):
        cfg.raise_mults[i] = m
    cfg.bet_allin = int(allin)
    cfg.bet_geometric = int(geo)
    cfg.max_raises = int(max_raises)
    return cfg


def make_spot(board: Sequence[int], oop: np.ndarray, ip: np.ndarray, pot: int,
              stack: int, filter_board: bool = True) -> _abi.Spot:
    sp = _abi.Spot()
    for i, c in enumerate(board):
        sp.board[i] = c
    sp.n_board = len(board)
    o = np.array(oop, dtype=np.float64)
    p = np.array(ip, dtype=np.float64)
    if filter_board:  # Range::filterBoard, as the reference binding does
        bset = set(board)
        for i in range(_abi.COMBOS):
            a, b = _combo_cards(i)
            if a in bset or b in bset:
                o[i] = 0.0
                p[i] = 0.0
    C.memmove(sp.oop, o.ctypes.data, o.nbytes)
    C.memmove(sp.ip, p.ctypes.data, p.nbytes)
    sp.pot = int(pot)
    sp.stack = int(stack)
    return sp


_COMBO_TABLE = [(a, b) for a in range(52) for b in range(a + 1, 52)]


def _combo_cards(i: int):
    return _COMBO_TABLE[i]


def _action(a: _abi.Action) -> Dict[str, Any]:
    return {"kind": _KIND.get(a.kind, "?"), "amount": int(a.amount)}


class Solver:
    """GPU postflop DCFR solver for one spot (reference: pps_native.Solver)."""

    def __init__(self, board: Any = None, oop: Any = None, ip: Any = None, pot: int = 0,
                 stack: int = 0, bets: Any = "0.75,a", raises: Any = "2.5,3",
                 max_raises: int = 0, streets: Optional[Sequence[Any]] = None,
                 _handle: Optional[int] = None):
        """``streets``: optional per-street configs [flop, turn, river], each a
        dict with keys bets / raises / max_raises (extension; the reference
        has one config for every street)."""
        self._h = C.c_void_p()
        if _handle is not None:
            self._h = C.c_void_p(_handle)
            return
        bd = parse_board(board)
        spot = make_spot(bd, _range_arg(oop), _range_arg(ip), pot, stack)
        if streets is None:
            cfg = _bet_config(bets, raises, max_raises)
            check(lib.pps_gb_create(C.byref(spot), C.byref(cfg), C.byref(self._h)))
        else:
            if len(streets) != 3:
                raise RuntimeError("streets must hold 3 configs (flop, turn, river)")
            arr = (_abi.BetConfig * 3)()
            for k, sc in enumerate(streets):
                arr[k] = _bet_config(sc.get("bets", bets), sc.get("raises", raises),
                                     sc.get("max_raises", max_raises))
            check(lib.pps_gb_create_streets(C.byref(spot), arr, C.byref(self._h)))

    @staticmethod
    def load(path: str) -> "Solver":
        h = C.c_void_p()
        check(lib.pps_gb_load(str(path).encode(), C.byref(h)))
        return Solver(_handle=h.value)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and h.value:
            lib.pps_gb_destroy(h)
            self._h = C.c_void_p()

    # -- solving --
    def solve(self, max_iters: int, algo: str = "dcfr", target: float = -1.0) -> None:
        check(lib.pps_gb_solve(self._h, int(max_iters), algo.encode(), float(target)))

    def continue_solve(self, max_iters: int, target: float = -1.0) -> None:
        check(lib.pps_gb_continue(self._h, int(max_iters), float(target)))

    def reset(self) -> None:
        check(lib.pps_gb_reset(self._h))

    def stats(self) -> Dict[str, Any]:
        st = _abi.NodeStats()
        check(lib.pps_gb_stats(self._h, C.byref(st)))
        return {"ev_oop": st.ev0, "ev_ip": st.ev1, "exploitability": st.expl,
                "pair_mass": int(st.pair_mass)}

    # -- properties --
    def info(self) -> _abi.Info:
        inf = _abi.Info()
        check(lib.pps_gb_get_info(self._h, C.byref(inf)))
        return inf

    @property
    def num_nodes(self) -> int:
        return self.info().num_nodes

    @property
    def max_depth(self) -> int:
        return self.info().max_depth

    @property
    def num_decide_nodes(self) -> int:
        return self.info().num_decide_nodes

    @property
    def iterations_run(self) -> int:
        return self.info().iterations_run

    @property
    def total_iterations(self) -> int:
        return int(self.info().total_iterations)

    # -- introspection / queries --
    def _decide(self, idx: int) -> _abi.DecideInfo:
        d = _abi.DecideInfo()
        check(lib.pps_gb_decide_node(self._h, int(idx), C.byref(d)))
        return d

    def decide_nodes(self) -> List[Dict[str, Any]]:
        out = []
        for i in range(self.num_decide_nodes):
            d = self._decide(i)
            out.append({"index": i, "node_id": d.node_id, "player": d.player,
                        "depth": d.depth, "n_board": d.n_board, "n_combos": d.n_combos,
                        "actions": [_action(d.actions[a]) for a in range(d.n_actions)],
                        "children": [int(d.children[a]) for a in range(d.n_actions)]})
        return out

    def _node_strategy(self, idx: int) -> np.ndarray:
        f = (C.c_double * _abi.MAX_ACTIONS)()
        n = C.c_int()
        check(lib.pps_gb_node_strategy(self._h, int(idx), f, C.byref(n)))
        return np.array(f[:n.value], dtype=np.float64)

    def root_strategy(self) -> np.ndarray:
        f = (C.c_double * _abi.MAX_ACTIONS)()
        n = C.c_int()
        check(lib.pps_gb_root_strategy(self._h, f, C.byref(n)))
        return np.array(f[:n.value], dtype=np.float64)

    def strategy(self, decide_idx: int = 0) -> Dict[str, Any]:
        na, nc = C.c_int(), C.c_int()
        acts = (_abi.Action * _abi.MAX_ACTIONS)()
        combos = (C.c_int * _abi.COMBOS)()
        freqs = np.zeros(_abi.MAX_ACTIONS * _abi.COMBOS, dtype=np.float64)
        check(lib.pps_gb_combo_strategy(self._h, int(decide_idx), C.byref(na), C.byref(nc),
                                        acts, combos,
                                        freqs.ctypes.data_as(C.POINTER(C.c_double))))
        d = self._decide(decide_idx)
        cards = self.player_cards(d.player)
        agg = self._node_strategy(decide_idx)
        cl = list(combos[:nc.value])
        out = {"index": int(decide_idx), "node_id": d.node_id, "player": d.player,
               "depth": d.depth,
               "actions": [_action(acts[a]) for a in range(na.value)],
               "cards": [card_text(cards[2 * c]) + card_text(cards[2 * c + 1]) for c in cl],
               "freqs": freqs[:na.value * nc.value].reshape(na.value, nc.value).copy(),
               "combos": cl}
        if agg.size:
            out["aggregate"] = agg
        return out

    def root_ev(self) -> Dict[str, Any]:
        out = {}
        for p, name in ((0, "oop"), (1, "ip")):
            n = C.c_int()
            combos = (C.c_int * _abi.COMBOS)()
            ev = np.zeros(_abi.COMBOS)
            mass = np.zeros(_abi.COMBOS)
            check(lib.pps_gb_root_ev(self._h, p, C.byref(n), combos,
                                     ev.ctypes.data_as(C.POINTER(C.c_double)),
                                     mass.ctypes.data_as(C.POINTER(C.c_double))))
            cards = self.player_cards(p)
            cl = list(combos[:n.value])
            out[name] = {"combos": cl,
                         "cards": [card_text(cards[2 * c]) + card_text(cards[2 * c + 1])
                                   for c in cl],
                         "ev": ev[:n.value].copy(), "mass": mass[:n.value].copy()}
        return out

    def node_ev(self, decide_idx: int = 0) -> Dict[str, Any]:
        dec, na = C.c_int(), C.c_int()
        acts = (_abi.Action * _abi.MAX_ACTIONS)()
        nc = (C.c_int * 2)()
        combos = (C.c_int * (2 * _abi.COMBOS))()
        ev = np.zeros(2 * _abi.COMBOS)
        mass = np.zeros(2 * _abi.COMBOS)
        agg = np.zeros(2)
        aev = np.zeros(_abi.MAX_ACTIONS * _abi.COMBOS)
        aagg = np.zeros(_abi.MAX_ACTIONS)
        dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
        check(lib.pps_gb_node_ev(self._h, int(decide_idx), C.byref(dec), C.byref(na), acts, nc,
                                 combos, dp(ev), dp(mass), dp(agg), dp(aev), dp(aagg)))
        out: Dict[str, Any] = {"decider": dec.value,
                               "actions": [_action(acts[a]) for a in range(na.value)]}
        ndec = nc[dec.value]
        out["action_ev"] = [{"per_combo": aev[a * _abi.COMBOS:a * _abi.COMBOS + ndec].copy(),
                             "agg_ev": float(aagg[a])} for a in range(na.value)]
        sides = {}
        for p, name in ((0, "oop"), (1, "ip")):
            cards = self.player_cards(p)
            b = p * _abi.COMBOS
            cl = list(combos[b:b + nc[p]])
            sides[name] = {"combos": cl,
                           "cards": [card_text(cards[2 * c]) + card_text(cards[2 * c + 1])
                                     for c in cl],
                           "ev": ev[b:b + nc[p]].copy(), "mass": mass[b:b + nc[p]].copy(),
                           "agg_ev": float(agg[p])}
        out["sides"] = sides
        return out

    def runout_summary(self, decide_idx: int, action_idx: int) -> Dict[str, Any]:
        dec, na, nb = C.c_int(), C.c_int(), C.c_int()
        acts = (_abi.Action * _abi.MAX_ACTIONS)()
        cards = (C.c_int * 52)()
        nxt = (C.c_int * 52)()
        nf = (C.c_int * 52)()
        freq = np.zeros(52 * _abi.MAX_ACTIONS)
        agg = np.zeros(104)
        check(lib.pps_gb_runout_summary(self._h, int(decide_idx), int(action_idx), C.byref(dec),
                                        C.byref(na), acts, C.byref(nb), cards, nxt, nf,
                                        freq.ctypes.data_as(C.POINTER(C.c_double)),
                                        agg.ctypes.data_as(C.POINTER(C.c_double))))
        brs = []
        for b in range(nb.value):
            brs.append({"card": card_text(cards[b]) if cards[b] >= 0 else "?",
                        "next_decide": int(nxt[b]),
                        "freq": freq[b * _abi.MAX_ACTIONS:b * _abi.MAX_ACTIONS + nf[b]].copy(),
                        "agg_ev": {"oop": float(agg[2 * b]), "ip": float(agg[2 * b + 1])}})
        return {"decider": dec.value, "actions": [_action(acts[a]) for a in range(na.value)],
                "branches": brs}

    def save(self, path: str, compressed: bool = False) -> None:
        """Writes a solution file; compressed=True stores the rows as 16-bit
        codes with one scale per action row (about half the size)."""
        fn = lib.pps_gb_save_compressed if compressed else lib.pps_gb_save
        check(fn(self._h, str(path).encode()))

    def player_cards(self, player: int) -> List[int]:
        buf = (C.c_uint8 * (2 * _abi.COMBOS))()
        n = C.c_int()
        check(lib.pps_gb_player_cards(self._h, int(player), buf, C.byref(n)))
        return list(buf[:2 * n.value])

    def player_weights(self, player: int) -> np.ndarray:
        w = np.zeros(_abi.COMBOS)
        n = C.c_int()
        check(lib.pps_gb_player_weights(self._h, int(player),
                                        w.ctypes.data_as(C.POINTER(C.c_double)), C.byref(n)))
        return w[:n.value].copy()

    def num_base_combos(self, player: int) -> int:
        return len(self.player_cards(player)) // 2

    def tree_structure(self) -> Dict[str, List[int]]:
        nn, nc = C.c_int(), C.c_int()
        check(lib.pps_gb_tree_structure(self._h, None, None, None, None, C.byref(nn),
                                        C.byref(nc)))
        kinds = (C.c_uint8 * max(nn.value, 1))()
        cb = (C.c_int * max(nn.value, 1))()
        ch = (C.c_int * max(nc.value, 1))()
        bd = (C.c_uint8 * max(5 * nn.value, 1))()
        check(lib.pps_gb_tree_structure(self._h, kinds, cb, ch, bd, C.byref(nn), C.byref(nc)))
        return {"kinds": list(kinds[:nn.value]), "child_base": list(cb[:nn.value]),
                "children": list(ch[:nc.value]), "boards": list(bd[:5 * nn.value])}

    # -- extension: rows, walks, engine choice (tests and benches) --
    def read_rows(self, which: int) -> np.ndarray:
        n = C.c_int64()
        check(lib.pps_gb_read_rows(self._h, int(which), None, 0, C.byref(n)))
        out = np.zeros(n.value, dtype=np.float32)
        check(lib.pps_gb_read_rows(self._h, int(which),
                                   out.ctypes.data_as(C.POINTER(C.c_float)), n.value,
                                   C.byref(n)))
        return out

    def write_rows(self, which: int, rows: np.ndarray) -> None:
        a = np.ascontiguousarray(rows, dtype=np.float32)
        check(lib.pps_gb_write_rows(self._h, int(which),
                                    a.ctypes.data_as(C.POINTER(C.c_float)), a.size))

    def walk(self, traverser: int, mode: int):
        """FP64 walk (mode 0 = EV vs the average strategy, 1 = best
        response); returns (root value in chips, root row)."""
        n = self.info().n_base[traverser]
        row = np.zeros(max(n, 1))
        v = C.c_double()
        check(lib.pps_gb_walk(self._h, int(traverser), int(mode),
                              row.ctypes.data_as(C.POINTER(C.c_double)), C.byref(v)))
        return v.value, row[:n].copy()

    def set_engine(self, kind: int) -> None:
        check(lib.pps_gb_set_engine(self._h, int(kind)))

    _SHAPE_KEYS = ("plan", "fwd_cap", "bwd_cap", "sd_cap", "fd_cap")

    def set_launch_shape(self, **shape: int) -> None:
        """Launch shape of the iteration graph (pps_gb_set_launch_shape):
        plan 0 / 2 and grid caps in SM multiples (0: one CTA per task);
        unnamed keys keep their current values. Turns the autotuner off."""
        cur = self.launch_shape()
        cur.update(shape)
        ls = _abi.LaunchShape(*[int(cur[k]) for k in self._SHAPE_KEYS])
        check(lib.pps_gb_set_launch_shape(self._h, C.byref(ls)))

    def launch_shape(self) -> Dict[str, int]:
        ls = _abi.LaunchShape()
        check(lib.pps_gb_get_launch_shape(self._h, C.byref(ls)))
        return {k: int(getattr(ls, k)) for k in self._SHAPE_KEYS}

    def set_compensated(self, on: bool = True) -> None:
        """Two-float cumulative-strategy sums (pps_gb_set_compensated)."""
        check(lib.pps_gb_set_compensated(self._h, 1 if on else 0))

    def time_iterations(self, n: int) -> float:
        """Milliseconds of n more iterations (graph replays, CUDA events on
        the solver's stream)."""
        ms = C.c_double()
        check(lib.pps_gb_time_iterations(self._h, int(n), C.byref(ms)))
        return ms.value

    def probe_bounded_wait(self, spins: int = 1024) -> None:
        """Diagnostic: a warp waits, bounded, for a copy that is never issued;
        raises the solver's device-wait error (PPS_GB_E_CUDA) afterwards."""
        check(lib.pps_gb_probe_bounded_wait(self._h, int(spins)))

    def profile(self, n: int, split_kinds: bool = False):
        """Per kernel class over n iterations: {name: (launches, ms, bytes)};
        split_kinds reports the backward pass per node kind."""
        out = (_abi.KernelStat * 16)()
        k = C.c_int()
        check(lib.pps_gb_profile(self._h, int(n), int(split_kinds), out, 16, C.byref(k)))
        return {out[i].name.decode(): (int(out[i].launches), out[i].ms, out[i].algo_bytes)
                for i in range(k.value)}

    def debug_dump(self) -> None:
        check(lib.pps_gb_debug_dump(self._h))


def compile_export(board: Sequence[int], oop: Any, ip: Any, pot: int, stack: int,
                   cfgs: Sequence[_abi.BetConfig]) -> Dict[str, np.ndarray]:
    """Host-only compile; returns the reference-layout artifacts by name."""
    dt = {b"i": np.int32, b"q": np.int64, b"B": np.uint8, b"f": np.float32, b"d": np.float64}
    out: Dict[str, np.ndarray] = {}

    def cb(_user, name, dtype, data, count):
        t = dt[dtype]
        if count:
            buf = C.string_at(data, count * np.dtype(t).itemsize)
            out[name.decode()] = np.frombuffer(buf, dtype=t).copy()
        else:
            out[name.decode()] = np.zeros(0, dtype=t)

    spot = make_spot(board, _range_arg(oop), _range_arg(ip), pot, stack, filter_board=False)
    arr = (_abi.BetConfig * len(cfgs))(*cfgs)
    check(lib.pps_gb_compile_export(C.byref(spot), arr, len(cfgs), _abi.ARRAY_CB(cb), None))
    return out


def layout_digest(board: Sequence[int], oop: Any, ip: Any, pot: int, stack: int,
                  cfgs: Sequence[_abi.BetConfig]) -> int:
    """Host-only: digest of the device layout built for the spot (tests)."""
    spot = make_spot(board, _range_arg(oop), _range_arg(ip), pot, stack, filter_board=False)
    arr = (_abi.BetConfig * len(cfgs))(*cfgs)
    d = C.c_uint64()
    check(lib.pps_gb_layout_digest(C.byref(spot), arr, len(cfgs), C.byref(d)))
    return int(d.value)


def bet_config(bets: Any, raises: Any, max_raises: int = 0) -> _abi.BetConfig:
    return _bet_config(bets, raises, max_raises)


def hand_keys(hands: np.ndarray) -> np.ndarray:
    h = np.ascontiguousarray(hands, dtype=np.uint8)
    keys = np.zeros(len(h), dtype=np.uint64)
    check(lib.pps_gb_hand_keys(h.ctypes.data_as(C.POINTER(C.c_uint8)), len(h),
                               keys.ctypes.data_as(C.POINTER(C.c_uint64))))
    return keys


def bet_actions(pot_base: int, stack: int, cfg: _abi.BetConfig, sc0: int, sc1: int, actor: int,
                after_allin: bool, num_bets: int, num_streets: int):
    out = (_abi.Action * _abi.MAX_ACTIONS)()
    n = C.c_int()
    check(lib.pps_gb_bet_actions(pot_base, stack, C.byref(cfg), sc0, sc1, actor,
                                 int(after_allin), num_bets, num_streets, out, C.byref(n)))
    return [(out[i].kind, int(out[i].amount)) for i in range(n.value)]
