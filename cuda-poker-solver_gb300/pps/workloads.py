"""Seeded synthetic spots for the solver's tests and benchmarks.

Every random draw comes from one documented generator, splitmix64 (Steele,
Lea, Flood 2014): state += 0x9E3779B97F4A7C15, then the two xor-shift-
multiply rounds; a uniform double is (x >> 11) * 2**-53. Boards draw
``next() % 52`` and reject repeats.

Named spots (pot/stack in chips, bets as pot fractions, "a" = all-in):

* ``river_c1``   river, both ranges all 1081 unblocked combos with weights
  U(0,1); pot 100, stack 100; bets {0.5, 1.0, a}, raises {2.0}, max 2.
* ``turn_c2``    turn, all 1128 combos U(0,1); pot 100, stack 200; turn bets
  {0.33, 0.75, a}, river bets {0.5, 1.0, a}, raises {2.5}, max 3 bets per
  street (per-street configs; ``turn_c2_uniform`` uses the turn config on
  both streets, the only form the reference can express).
* ``turn_c3``    turn, 60% of combos U(0.5,1) and the rest U(0,0.2); pot
  100, stack 400; bets {0.25, 0.5, 1.0, 1.5, a}, raises {2.0}, max 4
  (48,255 nodes).
* ``turn_w52``   the reference's own "wide" bench spot (tools/quality/
  bench_turn.sh:40-41): Qs9h2d7c, 300/1500, bets {0.25,0.5,0.75,1.25},
  raises {2.5,3.0}, ranges "22+,A9s+,KTs+,QJs,JTs,T9s" vs the same plus
  "AQo+" (51,903 nodes).
* ``flop_164k`` / ``flop_615k``  the reference's flop bench spots
  (docs/STATUS.md:75-84): Qs9h2d, bets {0.75, a}, raises {2.5, 3}, the
  wide ranges; pot/stack 200/500 (164,416 nodes) and 300/1500 (615,234).
* ``flop_wide``  the reference's 11,716,550-node flop (docs/STATUS.md:76):
  Qs9h2d, 300/1500, bets {0.25, 0.5, 0.75, 1.25}, raises {2.5, 3}.
* ``turn_api``   the reference's API test spot (python/test_pps.py:18-24).
* ``turn_tiny``  the reference's known-answer spot (tools/tiny_check.cpp:
  75-79, driven by tools/quality/gpu_postflop_parity.sh:139).
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Optional
import math

MASK64 = (1 << 64) - 1
RANKS = "23456789TJQKA"
SUITS = "cdhs"


class SplitMix64:
    def __init__(self, seed: int):
        self.state = seed & MASK64

    def next(self) -> int:
        self.state = (self.state + 0x9E3779B97F4A7C15) & MASK64
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
        return z ^ (z >> 31)

    def uniform(self) -> float:
        return (self.next() >> 11) * (2.0 ** -53)


def card_id(text: str) -> int:
    return SUITS.index(text[1].lower()) * 13 + RANKS.index(text[0].upper())


def card_text(cid: int) -> str:
    return RANKS[cid % 13] + SUITS[cid // 13]


def board_ids(text: str) -> List[int]:
    return [card_id(text[i:i + 2]) for i in range(0, len(text), 2)]


def draw_board(rng: SplitMix64, n: int) -> List[int]:
    out: List[int] = []
    while len(out) < n:
        c = rng.next() % 52
        if c not in out:
            out.append(c)
    return out


@dataclass
class BetCfg:
    """pf::BetConfig (src/postflop_cfr.h:24-42)."""
    bets: List[float] = field(default_factory=list)
    raises: List[float] = field(default_factory=list)
    allin: bool = False
    geometric: bool = False
    max_raises: int = 0
    add_allin: float = 1.5
    force_allin: float = 0.15
    merging: float = 0.1

    def bet_text(self) -> str:
        toks = ["%g" % b for b in self.bets]
        if self.allin:
            toks.append("a")
        if self.geometric:
            toks.append("e")
        return ",".join(toks)

    def raise_text(self) -> str:
        return ",".join("%g" % r for r in self.raises)


@dataclass
class Spot:
    name: str
    board: List[int]
    oop: object            # 1326 weights (list) or a range string
    ip: object
    pot: int
    stack: int
    cfg: BetCfg
    street_cfgs: Optional[List[BetCfg]] = None  # [flop, turn, river]
    iterations: int = 1000

    def board_text(self) -> str:
        return "".join(card_text(c) for c in self.board)


def uniform_weights(rng: SplitMix64) -> List[float]:
    return [rng.uniform() for _ in range(1326)]


def mixture_weights(rng: SplitMix64) -> List[float]:
    out = []
    for _ in range(1326):
        if rng.uniform() < 0.6:
            out.append(0.5 + 0.5 * rng.uniform())
        else:
            out.append(0.2 * rng.uniform())
    return out


def river_c1(seed: int = 101) -> Spot:
    rng = SplitMix64(seed)
    board = draw_board(rng, 5)
    return Spot("river_c1", board, uniform_weights(rng), uniform_weights(rng),
                100, 100, BetCfg([0.5, 1.0], [2.0], allin=True, max_raises=2),
                iterations=1000)


def turn_c2(seed: int = 202, uniform_config: bool = False) -> Spot:
    rng = SplitMix64(seed)
    board = draw_board(rng, 4)
    turn = BetCfg([0.33, 0.75], [2.5], allin=True, max_raises=3)
    river = BetCfg([0.5, 1.0], [2.5], allin=True, max_raises=3)
    s = Spot("turn_c2", board, uniform_weights(rng), uniform_weights(rng),
             100, 200, turn, [turn, turn, river], iterations=500)
    if uniform_config:
        s.name = "turn_c2_uniform"
        s.street_cfgs = None
    return s


def turn_c3(seed: int = 303) -> Spot:
    rng = SplitMix64(seed)
    board = draw_board(rng, 4)
    return Spot("turn_c3", board, mixture_weights(rng), mixture_weights(rng),
                100, 400,
                BetCfg([0.25, 0.5, 1.0, 1.5], [2.0], allin=True, max_raises=4),
                iterations=1000)


def turn_w52() -> Spot:
    return Spot("turn_w52", board_ids("Qs9h2d7c"), "22+,A9s+,KTs+,QJs,JTs,T9s",
                "22+,A9s+,KTs+,QJs,JTs,T9s,AQo+", 300, 1500,
                BetCfg([0.25, 0.5, 0.75, 1.25], [2.5, 3.0]), iterations=2000)


def flop_164k() -> Spot:
    """The reference's practical flop abstraction (docs/STATUS.md:81-84):
    Qs9h2d, pot 200, stack 500, bets {0.75, a}, raises {2.5, 3}, the wide
    bench ranges (164,416 nodes; ~201 it/s on the reference's RTX 4070)."""
    return Spot("flop_164k", board_ids("Qs9h2d"), "22+,A9s+,KTs+,QJs,JTs,T9s",
                "22+,A9s+,KTs+,QJs,JTs,T9s,AQo+", 200, 500,
                BetCfg([0.75], [2.5, 3.0], allin=True), iterations=200)


def flop_615k() -> Spot:
    """The same abstraction at pot 300, stack 1500 (615,234 nodes; the
    reference's "flop standard", ~55 it/s, docs/STATUS.md:75)."""
    return Spot("flop_615k", board_ids("Qs9h2d"), "22+,A9s+,KTs+,QJs,JTs,T9s",
                "22+,A9s+,KTs+,QJs,JTs,T9s,AQo+", 300, 1500,
                BetCfg([0.75], [2.5, 3.0], allin=True), iterations=200)


def flop_wide() -> Spot:
    """The reference's "flop wide" spot (docs/STATUS.md:76): Qs9h2d,
    300/1500, bets {0.25, 0.5, 0.75, 1.25}, raises {2.5, 3}, the wide
    ranges (11,716,550 nodes; ~0.57 it/s on the reference's RTX 4070)."""
    return Spot("flop_wide", board_ids("Qs9h2d"), "22+,A9s+,KTs+,QJs,JTs,T9s",
                "22+,A9s+,KTs+,QJs,JTs,T9s,AQo+", 300, 1500,
                BetCfg([0.25, 0.5, 0.75, 1.25], [2.5, 3.0]), iterations=100)


def turn_api() -> Spot:
    return Spot("turn_api", board_ids("Qs9h2d7c"), "TT+,AKo", "AQ+,KQs", 200,
                500, BetCfg([0.75], [2.5, 3.0], allin=True), iterations=300)


def turn_tiny() -> Spot:
    return Spot("turn_tiny", board_ids("Qs9h2d7c"), "TT+", "99+", 200, 3000,
                BetCfg([0.5], []), iterations=0)


def batched(count: int = 256, seed: int = 404) -> List[Spot]:
    """The batched/served distribution: 70% river / 30% turn spots, weights
    U(0,1), pot U(50,200), stack/pot log-uniform in [1, 8], 2-4 bet sizes
    from {25,33,50,75,100,150}% plus all-in, raises {2.5}, max 3."""
    rng = SplitMix64(seed)
    sizes = [0.25, 0.33, 0.5, 0.75, 1.0, 1.5]
    out = []
    for k in range(count):
        river = rng.uniform() < 0.7
        board = draw_board(rng, 5 if river else 4)
        pot = 50 + int(150 * rng.uniform())
        spr = math.exp(math.log(8.0) * rng.uniform())
        stack = max(1, int(round(pot * spr)))
        n_sizes = 2 + int(3 * rng.uniform())
        pool = list(sizes)
        chosen = []
        for _ in range(min(n_sizes, 4)):
            chosen.append(pool.pop(rng.next() % len(pool)))
        chosen.sort()
        out.append(Spot("batch_%03d" % k, board, uniform_weights(rng),
                        uniform_weights(rng), pot, stack,
                        BetCfg(chosen, [2.5], allin=True, max_raises=3),
                        iterations=1000))
    return out


def c3_stream(count: int = 1024, seed: int = 606) -> List[Spot]:
    """The served distribution: spots drawn like turn_c3 (48,255-node turn
    trees), each with its own seeded 4-card board and mixture ranges (60%
    of combos at U(0.5, 1), the rest U(0, 0.2)); pot 100, stack 400, bets
    {25, 50, 100, 150}% plus all-in on both streets, raises 2x, max 4."""
    return [turn_c3(seed=seed * 1000003 + k) for k in range(count)]


def turn_short() -> Spot:
    """Short stack: all-in on the turn, the river is a dead-street runout
    (the regression spot of tools/quality/gpu_postflop_parity.sh:139)."""
    a = turn_api()
    return Spot("turn_short", a.board, a.oop, a.ip, 500, 150, BetCfg([0.5, 0.75], [2.5, 3.0]))


def flop_short() -> Spot:
    return Spot("flop_short", board_ids("Qs9h2d"), "AA,KK", "QQ,JJ,AKs", 100, 40,
                BetCfg([0.5], [], max_raises=1))


def flop_small() -> Spot:
    return Spot("flop_small", board_ids("Qs9h2d"), "AA,KK", "QQ,JJ,AKs", 100, 100,
                BetCfg([0.5], [], max_raises=1))


def river_geo() -> Spot:
    return Spot("river_geo", board_ids("Qs9h2d7c3h"), "TT+,AKo,KQs", "99+,AJs+,KQo", 100, 450,
                BetCfg([0.33], [2.0], allin=True, geometric=True, max_raises=2))


def river_empty() -> Spot:
    return Spot("river_empty", board_ids("AsAhAdKsKh"), "AA", "KK,QQ", 100, 100,
                BetCfg([0.5], []))


NAMED = {
    "river_c1": river_c1,
    "turn_c2": turn_c2,
    "turn_c2_uniform": lambda: turn_c2(uniform_config=True),
    "turn_c3": turn_c3,
    "turn_w52": turn_w52,
    "flop_164k": flop_164k,
    "flop_615k": flop_615k,
    "flop_wide": flop_wide,
    "turn_api": turn_api,
    "turn_tiny": turn_tiny,
    "turn_short": turn_short,
    "flop_short": flop_short,
    "flop_small": flop_small,
    "river_geo": river_geo,
    "river_empty": river_empty,
}
