"""Leveled kernels: a time-series stage split into time-parallel and scan kernels.

The reference walks every stage sequentially over time, one stock block per
task (``KunQuant/passes/CodegenCpp.py:189``).  Most ops do not need that: a
back-window loop's output at time t depends only on the window's values, and
the order-statistic window of the skip-list ops is fully determined by the
last W values.  Only the history-dependent states -- Kahan running sums
(``FastWindowedSum``), the regression sums (``WindowedLinearRegression``) and
``ExpMovingAvg`` -- need a sequential scan from the first row.

Each op of a stage gets a *level*.  Even levels are time-parallel kernels (one
thread per stock x time chunk, no carried state; order-statistic windows are
rebuilt exactly with a W-row warm-up).  Odd levels are scan kernels: one thread
per stock x state walks the whole time axis and stores the state's per-row
result.  Values that cross levels are materialised in [T][S] scratch buffers;
cheap pointwise ops are recomputed where they are needed.  A windowed read
(loop, BackRef, skip list, running sum) only reads series materialised at an
earlier level, so every kernel reads exactly the values the sequential
reference computes and the arithmetic of every op is unchanged.
"""
from typing import Dict, List, Optional, Set, Tuple

from . import contraction

SEQ = {"FastWindowedSum", "WindowedLinearRegression", "ExpMovingAvg", "SlideReduce"}
# states that depend on the last `window` rows only: a scan over them can
# start anywhere with a warm-up of one window (time-chunked scans)
FINITE_SEQ = {"FastWindowedSum", "WindowedLinearRegression", "SlideReduce"}
UNSUPPORTED: Set[str] = set()
ACC = {"Accumulator", "SetAccumulator"}
LR_CONS = {"WindowedLinearRegressionRSqaureImpl", "WindowedLinearRegressionSlopeImpl",
           "WindowedLinearRegressionResiImpl"}
SL_CONS = {"SkipListQuantile", "SkipListRank", "SkipListMin", "SkipListMax", "SkipListArgMin"}
REDUCTIONS = {"ReduceAdd", "ReduceMul", "ReduceMin", "ReduceMax", "ReduceArgMax",
              "ReduceArgMin", "ReduceRank", "ReduceDecayLinear"}
ANCHORS = SEQ | LR_CONS | SL_CONS | REDUCTIONS | ACC | {"WindowedTempOutput", "Output", "SkipListState",
                                                        "ForeachBackWindow"}


def _even_ge(x: int) -> int:
    x = max(x, 0)
    return x if x % 2 == 0 else x + 1


def _odd_ge(x: int) -> int:
    x = max(x, 1)
    return x if x % 2 == 1 else x + 1


class Unsupported(Exception):
    pass


class StagePlan:
    """Level assignment of one time-series stage."""

    def __init__(self, ops: List[dict], plain: bool = False):
        self.ops = ops
        self.plain = plain
        self.fused_products: Set[int] = set()
        n = len(ops)
        for op in ops:
            if op["k"] in UNSUPPORTED:
                raise Unsupported(op["k"])
            if op["k"] == "ForeachBackWindow" and op.get("p", -1) >= 0:
                raise Unsupported("nested loop")
        self.lv: List[int] = [-1] * n
        self.loop_chain: Dict[int, List[int]] = {}
        self._chains()
        self._acc_groups()
        self._assign()
        if plain:
            self._assign_plain()

    # Accumulator recurrences (the fast-stat rolling moments): an
    # Accumulator's value at row t is what its SetAccumulator stored at row
    # t-1.  The ops between the reads and the sets of coupled accumulators
    # form one group that a scan kernel walks through time; every other op
    # that reads a group value does so from memory at a later level.
    def _acc_groups(self):
        ops = self.ops
        n = len(ops)
        dep = [False] * n  # depends on some accumulator's value
        for i, op in enumerate(ops):
            if op["k"] == "Accumulator" or any(dep[j] for j in op["in"]):
                dep[i] = True
                if op.get("p", -1) >= 0:
                    raise Unsupported("accumulator value used inside a loop")
        self.state_dep = dep
        parent = {i: i for i, op in enumerate(ops) if op["k"] == "Accumulator"}

        def find(x):
            while parent[x] != x:
                parent[x] = parent[parent[x]]
                x = parent[x]
            return x

        on_path: Dict[int, Set[int]] = {}
        for i, op in enumerate(ops):
            if op["k"] != "SetAccumulator":
                continue
            acc = op["in"][0]
            # state-dependent ops on the way back from the set to the reads
            seen, stack = set(), list(op["in"][1:])
            while stack:
                j = stack.pop()
                if j in seen or not dep[j]:
                    continue
                seen.add(j)
                if ops[j]["k"] == "Accumulator":
                    parent[find(j)] = find(acc)
                    continue
                stack.extend(ops[j]["in"])
            on_path[i] = seen | {i, acc}
        groups: Dict[int, Set[int]] = {}
        for i, mem in on_path.items():
            groups.setdefault(find(ops[i]["in"][0]), set()).update(mem)
        for a in parent:
            groups.setdefault(find(a), set()).add(a)
        for mem in groups.values():
            for j in mem:
                ws = self.windowed_source(j)
                if ops[j]["k"] == "WindowedTempOutput" or (ws is not None and dep[ws]):
                    # a statistic over a statistic: the inner values would have
                    # to be written and read back inside the same scan
                    raise Unsupported("windowed read of a group value inside the group")
        self.acc_group: Dict[int, int] = {}
        self.groups: Dict[int, Set[int]] = groups
        for g, mem in groups.items():
            for j in mem:
                self.acc_group[j] = g

    # loops merged by merge_loops share reductions: they form one chain
    def _chains(self):
        ops = self.ops
        chain: List[int] = []
        for i, op in enumerate(ops):
            if op["k"] != "ForeachBackWindow":
                continue
            if op.get("copy_prev_body") and chain:
                chain.append(i)
            else:
                chain = [i]
            for j in chain:
                self.loop_chain[j] = chain

    def body(self, loop: int) -> List[int]:
        return [j for j, o in enumerate(self.ops) if o.get("p", -1) == loop]

    def windowed_source(self, i: int) -> Optional[int]:
        op = self.ops[i]
        k = op["k"]
        if k in ("FastWindowedSum", "WindowedLinearRegression", "BackRef"):
            return op["in"][0]
        if k == "SlideReduce":
            return op["in"][0]
        if k == "IterValue":
            return op["in"][1]
        if k == "SkipListState":
            return self.ops[op["in"][0]]["in"][0]
        return None

    def _assign(self):
        ops, lv = self.ops, self.lv
        self._done_chain = set()
        windowed_outputs = set()
        for i, op in enumerate(ops):
            ws = self.windowed_source(i)
            if ws is not None and ops[ws]["k"] == "Output":
                windowed_outputs.add(ws)
            if op["k"] == "SlideReduce":
                windowed_outputs |= {j for j in op["in"][:op["nsrc"]] if ops[j]["k"] == "Output"}
        self._windowed_outputs = windowed_outputs
        # ops that do not depend on accumulator values first; then each
        # accumulator group goes to the first scan level after its inputs,
        # then the readers of group values
        dep = self.state_dep
        for i in range(len(ops)):
            if not dep[i]:
                self._assign_op(i)
        # a group can read values derived from another group: iterate until
        # the levels settle (the groups form a DAG)
        self.group_level: Dict[int, int] = {}
        for _ in range(len(self.groups) + 2):
            changed = False
            for g, mem in self.groups.items():
                ext = []
                for j in mem:
                    if ops[j]["k"] == "Accumulator":
                        continue
                    for x in ops[j]["in"]:
                        if x not in mem:
                            if dep[x]:
                                raise Unsupported("accumulator group reads another group's values")
                            ext.append(self._vl(x))
                base = max(ext + [-1])
                L = _odd_ge(base + 1 if base % 2 == 1 else base)
                if self.group_level.get(g) != L:
                    self.group_level[g] = L
                    changed = True
            for i in range(len(ops)):
                if dep[i]:
                    if i in self.acc_group:
                        lv[i] = self.group_level[self.acc_group[i]]
                    else:
                        self._assign_op(i)
            if not changed:
                break
        else:
            raise Unsupported("accumulator groups do not settle")
        self._finish_levels()

    def _assign_op(self, i: int):
        ops, lv = self.ops, self.lv
        done_chain = self._done_chain
        windowed_outputs = self._windowed_outputs
        if True:
            op = ops[i]
            k = op["k"]
            ins = op["in"]
            if op.get("p", -1) >= 0:
                return
            if k in ("Input", "ConstantOp"):
                lv[i] = -1
            elif k in ("FastWindowedSum", "WindowedLinearRegression"):
                src = ins[0]
                lv[i] = _odd_ge(lv[src] + 1 if lv[src] >= 0 else 0)
            elif k == "ExpMovingAvg":
                lv[i] = _odd_ge(max(lv[j] for j in ins))
            elif k == "SlideReduce":
                # window reads of materialised sources, invariants at row t
                ns = op["nsrc"]
                base = max([lv[j] + 1 if lv[j] >= 0 else 0 for j in ins[:ns]] +
                           [self._vl(j) for j in ins[ns:]] + [0])
                lv[i] = _odd_ge(base)
            elif k in LR_CONS:
                lv[i] = lv[ins[0]]
                if any(lv[j] > lv[i] for j in ins[1:]):
                    raise Unsupported("regression residual of a later value")
            elif k == "SkipListState":
                src = self.windowed_source(i)
                if ins[1] != src:
                    raise Unsupported("skip list over a different current value")
                lv[i] = _even_ge(lv[src] + 1 if lv[src] >= 0 else 0)
            elif k in SL_CONS:
                lv[i] = lv[ins[0]]
                if any(lv[j] > lv[i] for j in ins[1:]):
                    raise Unsupported("skip-list rank of a later value")
            elif k == "WindowedTempOutput":
                lv[i] = _even_ge(lv[ins[0]])
            elif k == "ForeachBackWindow":
                chain = self.loop_chain[i]
                if chain[0] not in done_chain:
                    base = 0
                    for lp in chain:
                        for j in self.body(lp):
                            bo = ops[j]
                            if bo["k"] == "IterValue":
                                s = bo["in"][1]
                                base = max(base, lv[s] + 1 if lv[s] >= 0 else 0)
                            else:
                                for x in bo["in"]:
                                    if ops[x].get("p", -1) < 0 and ops[x]["k"] != "ForeachBackWindow":
                                        base = max(base, lv[x])
                    for j, q in enumerate(ops):
                        if q["k"] == "ReduceRank" and contraction.reduction_loop(ops, j) in chain:
                            base = max(base, lv[q["in"][1]])
                    L = _even_ge(base)
                    for lp in chain:
                        lv[lp] = L
                        for j in self.body(lp):
                            lv[j] = L
                    done_chain.add(chain[0])
            elif k in REDUCTIONS:
                lv[i] = lv[contraction.reduction_loop(ops, i)]
            elif k == "BackRef":
                src = ins[0]
                lv[i] = lv[src] + 1 if lv[src] >= 0 else -1
            elif k == "Output":
                lv[i] = _even_ge(lv[ins[0]]) if i in windowed_outputs else None
            else:
                lv[i] = max([self._vl(j) for j in ins] + [-1])

    def _finish_levels(self):
        ops, lv = self.ops, self.lv
        # outputs not read back in the stage go to the last parallel level
        top = max([x for x in lv if x is not None] + [0])
        final = _even_ge(top)
        for i, op in enumerate(ops):
            if op["k"] == "Output" and lv[i] is None:
                lv[i] = final
        self.final = final
        self.levels = sorted({lv[i] for i, op in enumerate(ops)
                              if op["k"] in ANCHORS and op.get("p", -1) < 0 and lv[i] >= 0})
        if not self.levels:
            self.levels = [0]

    def _vl(self, j: int) -> int:
        while self.lv[j] is None:
            j = self.ops[j]["in"][0]
        return self.lv[j]

    def is_anchor(self, i: int) -> bool:
        op = self.ops[i]
        if op.get("p", -1) >= 0:
            return False
        if self.plain:
            return op["k"] not in ("Input", "ConstantOp") and i not in self.fused_products
        return op["k"] in ANCHORS

    # One launch per op (the baseline form): every op that is not a source gets
    # a level of its own and its value goes through memory.  Ops that share
    # state stay together: a loop with its body and reductions, a regression
    # or an order-statistic window with its readers, an accumulator group.
    def _assign_plain(self):
        ops, lv = self.ops, self.lv
        # a product contracted into its adder is recomputed by the adder
        self.fused_products = {prod for _, (_, prod) in contraction.plan(ops).items()}
        unit_of: Dict[int, int] = {}
        for i, op in enumerate(ops):
            k = op["k"]
            if op.get("p", -1) >= 0:
                continue
            if k in ("Input", "ConstantOp") or i in self.fused_products:
                continue
            if k == "ForeachBackWindow":
                unit_of[i] = self.loop_chain[i][0]
            elif k in REDUCTIONS:
                unit_of[i] = self.loop_chain[contraction.reduction_loop(ops, i)][0]
            elif k in LR_CONS or k in SL_CONS:
                unit_of[i] = op["in"][0]
            elif i in self.acc_group:
                unit_of[i] = ("g", self.acc_group[i])
            else:
                unit_of[i] = i
        members: Dict[object, List[int]] = {}
        for i, u in unit_of.items():
            members.setdefault(u, []).append(i)
        for lp, chain in self.loop_chain.items():
            if chain[0] == lp:
                for c in chain:
                    members[chain[0]] += [j for j in self.body(c) if j not in members[chain[0]]]
        seq = lambda u: (isinstance(u, tuple) or ops[u]["k"] in SEQ)  # noqa: E731
        ext: Dict[object, Set[int]] = {}
        for u, mem in members.items():
            ms = set(mem)
            e = set()
            stack = [x for j in mem if ops[j]["k"] != "Accumulator" for x in ops[j]["in"]]
            while stack:
                x = stack.pop()
                if x in ms:
                    continue
                if x in self.fused_products:
                    stack.extend(ops[x]["in"])
                elif x in unit_of and unit_of[x] != u:
                    e.add(x)
            ext[u] = e
        done: Dict[object, int] = {}
        cur = -1
        pending = sorted(members, key=lambda u: max(members[u]))
        while pending:
            progress = False
            for u in list(pending):
                if any(unit_of[x] not in done for x in ext[u]):
                    continue
                L = cur + 1
                if seq(u) != (L % 2 == 1):
                    L += 1
                cur = L
                done[u] = L
                for j in members[u]:
                    lv[j] = L
                pending.remove(u)
                progress = True
            if not progress:
                raise Unsupported("plain form: cyclic units")
        self.levels = sorted(set(done.values())) or [0]
        self.final = max(self.levels)

    def is_source(self, i: int) -> bool:
        return self.ops[i]["k"] in ("Input", "ConstantOp")

    # ---------------------------------------------------------------- sets
    def chain_members(self, loop: int) -> List[int]:
        """All ops of the loop chain of `loop`: loops, body ops, reductions."""
        ops = self.ops
        chain = self.loop_chain[loop]
        out = list(chain)
        for lp in chain:
            out += self.body(lp)
        for j, q in enumerate(ops):
            if q["k"] in REDUCTIONS and contraction.reduction_loop(ops, j) in chain:
                out.append(j)
        return out

    def value_source(self, j: int, level: int) -> int:
        """Outputs and windowed temps are copies of their input; when they are
        materialised later than `level`, their input is used instead."""
        ops = self.ops
        while ops[j]["k"] in ("Output", "WindowedTempOutput") and self.lv[j] > level:
            j = ops[j]["in"][0]
        return j

    def closure(self, roots: List[int], level: int) -> Tuple[Set[int], Set[int], Set[int]]:
        """(ops computed at `level` for `roots`, ops whose value is read from
        memory, series read through windows)."""
        ops, lv = self.ops, self.lv
        comp: Set[int] = set()
        vreads: Set[int] = set()
        wreads: Set[int] = set()
        stack = list(roots)
        while stack:
            i = stack.pop()
            if i in comp:
                continue
            op = ops[i]
            k = op["k"]
            if k == "Input":
                vreads.add(i)
                continue
            if self.is_anchor(i) and k != "ForeachBackWindow" and op.get("p", -1) < 0 and lv[i] < level:
                vreads.add(i)
                continue
            if self.is_anchor(i) and op.get("p", -1) < 0 and lv[i] > level:
                raise Unsupported(f"op {i} ({k}) of level {lv[i]} needed at level {level}")
            comp.add(i)
            loop = None
            if k == "ForeachBackWindow":
                loop = i
            elif k in REDUCTIONS:
                loop = contraction.reduction_loop(ops, i)
            elif op.get("p", -1) >= 0:
                loop = op["p"]
            if loop is not None:
                for j in self.chain_members(loop):
                    if j not in comp:
                        stack.append(j)
            deps: List[int] = []
            if k == "IterValue":
                wreads.add(op["in"][1])
            elif k == "ForeachBackWindow":
                pass
            elif k in REDUCTIONS:
                deps = op["in"][1:]
            elif k == "BackRef":
                wreads.add(op["in"][0])
            elif k in ("FastWindowedSum", "WindowedLinearRegression"):
                wreads.add(op["in"][0])
                deps = [op["in"][0]]
            elif k == "SlideReduce":
                wreads |= set(op["in"][:op["nsrc"]])
                deps = list(op["in"])
            elif k == "Accumulator":
                deps = []  # its input only orders it; the value is the state
            elif k == "SkipListState":
                wreads.add(self.windowed_source(i))
                deps = list(op["in"])
            else:
                deps = list(op["in"])
            for d in deps:
                if ops[d].get("p", -1) >= 0 and op.get("p", -1) < 0:
                    continue
                stack.append(self.value_source(d, level) if ops[d].get("p", -1) < 0 else d)
        return comp, vreads, wreads


# ====================================================================== codegen
from .codegen import StageGen  # noqa: E402

PAR_CHUNK = 32
REG_WINDOW_MAX = 64
VEC_U = 4
# rows a thread computes at once in a kernel without window loops, where
# the rows share no loads and more of them only cost registers
VEC_U_ELEM = 2
# rows a window queue loads ahead of use, and the unroll of the window loop
VEC_PREFETCH = 0
VEC_UNROLL = 4
SCAN_BLOCK = 16
# window sums (two floats each) one chunked scan of the slide form keeps
SLIDE_MAX_SUMS = 10
# rows a chunked scan of the slide form loads at once
SLIDE_BLOCK = 2
WIDE_SERIES = 24


class LeveledGen(StageGen):
    """Emits the leveled kernels of one time-series stage."""

    def __init__(self, spec: dict, si: int, tag: str):
        super().__init__(spec, si, tag)
        self.plan = StagePlan(self.ops, plain=spec.get("form") == "plain")
        self.fplan = contraction.plan(self.ops)
        # sliding-moment form: running sums as deduplicated two-float window
        # sums, scans in time chunks (see slide.py)
        self.slide = spec.get("form") == "slide"
        self.chunk_mode = False
        # staged (TMA) instance of an elementwise kernel being generated:
        # series -> stage index; store_guard keeps threads past the last
        # stock from storing
        self.tma_slot: Optional[Dict[int, int]] = None
        self.store_guard = ""
        self.tma_kernels: Dict[int, List[str]] = {}
        self.mom: Dict[tuple, str] = {}
        self.cur_level = None
        self.cur_comp: Set[int] = set()
        self.vec = False
        self.pf_window = None
        self.mats: Set[int] = set()

    def val(self, i: int) -> str:
        if self.cur_level is not None and self.ops[i].get("p", -1) < 0:
            i = self.plan.value_source(i, self.cur_level)
        top = self.ops[i].get("p", -1) < 0
        if self.ops[i]["k"] in REDUCTIONS and i not in self.cur_comp:
            return f"v{i}[u]" if self.vec else f"v{i}"  # materialised earlier, loaded per row
        if self.vec and top:
            if self.ops[i]["k"] in REDUCTIONS:
                return self.reduction_value(i, f"r{i}[u]")
            return f"v{i}[u]"
        return super().val(i)

    # ------------------------------------------------------------------ memory
    def _kernels(self):
        plan, ops, lv = self.plan, self.ops, self.plan.lv
        ks = []
        prev_cscans: List[dict] = []
        for L in plan.levels:
            if L % 2 == 0:
                roots = [i for i in range(len(ops)) if plan.is_anchor(i) and lv[i] == L
                         and ops[i]["k"] not in SEQ]
                if self.slide and prev_cscans:
                    roots = self._fuse_into_scans(roots, L, prev_cscans)
                prev_cscans = []
                if roots:
                    for role in self._par_roles(roots, L):
                        ks.append(dict(role, level=L, kind="par"))
            else:
                roles = []
                for i in range(len(ops)):
                    if ops[i]["k"] in SEQ and lv[i] == L:
                        roots = [i] + [j for j, q in enumerate(ops) if q["k"] in LR_CONS and q["in"][0] == i]
                        comp, vr, wr = plan.closure(roots, L)
                        roles.append({"roots": roots, "comp": comp, "vr": vr, "wr": wr})
                for g, mem in sorted(plan.groups.items()):
                    if plan.group_level[g] != L:
                        continue
                    roots = sorted(j for j in mem if ops[j]["k"] in ACC)
                    comp, vr, wr = plan.closure(roots, L)
                    roles.append({"roots": roots, "comp": comp, "vr": vr, "wr": wr})
                prev_cscans = []
                if roles and self.slide:
                    whole = []
                    for r in self._slide_roles(roles, L):
                        if self._chunkable(r):
                            ks.append({"level": L, "kind": "cscan", "roles": [r]})
                            prev_cscans.append(r)
                        else:
                            whole.append(r)
                    roles = whole
                if roles:
                    ks.append({"level": L, "kind": "scan", "roles": roles})
        return ks

    def _fuse_into_scans(self, roots: List[int], L: int, scans: List[dict]) -> List[int]:
        """Slide form: an output of level L that is a pointwise function of
        one chunked scan's values (of level L - 1) and of series already in
        memory is computed and stored by that scan, so the scan's values are
        not written to memory and read back.  Returns the roots left."""
        plan, ops, lv = self.plan, self.ops, self.plan.lv
        left = []
        for r in roots:
            target = None
            if ops[r]["k"] == "Output" and r not in self.plan._windowed_outputs:
                try:
                    comp, vr, wr = plan.closure([r], L)
                except Unsupported:
                    comp, vr, wr = set(), set(), {None}
                pointwise = not wr and all(j == r or not plan.is_anchor(j) for j in comp)
                need = {j for j in vr if lv[j] == L - 1}
                if pointwise and need:
                    for sc in scans:
                        if need <= sc["comp"]:
                            target = sc
                            break
            if target is None:
                left.append(r)
                continue
            lv[r] = L - 1
            target["roots"] = sorted(set(target["roots"]) | {r})
            target["comp"], target["vr"], target["wr"] = plan.closure(target["roots"], L - 1)
        return left

    def _chunkable(self, role: dict) -> bool:
        """A scan role whose states all forget rows older than their window
        runs in time chunks, each starting one window early."""
        ops = self.ops
        return all(ops[i]["k"] in FINITE_SEQ for i in role["comp"] if ops[i]["k"] in SEQ | ACC)

    def _slide_roles(self, roles: List[dict], L: int) -> List[dict]:
        """Scan roles of the slide form merged when they read a common
        series through a window: the window sums over the same series share
        their loads, and sums that several roles need (a mean that is also
        an invariant of a moment) are kept once.  A merged role holds at most
        SLIDE_MAX_SUMS window sums (registers)."""
        ops, plan = self.ops, self.plan
        items = []
        rest = []
        for r in roles:
            seqs = [i for i in r["roots"] if ops[i]["k"] in FINITE_SEQ]
            if len(seqs) != 1 or ops[seqs[0]]["k"] == "WindowedLinearRegression":
                rest.append(r)
                continue
            op = ops[seqs[0]]
            srcs = op["in"][:op["nsrc"]] if op["k"] == "SlideReduce" else op["in"][:1]
            items.append((set(srcs), op["window"], r))
        parent = list(range(len(items)))

        def find(x):
            while parent[x] != x:
                parent[x] = parent[parent[x]]
                x = parent[x]
            return x

        for a in range(len(items)):
            for b in range(a):
                if items[a][0] & items[b][0]:
                    parent[find(a)] = find(b)
        groups: Dict[int, list] = {}
        for a in range(len(items)):
            groups.setdefault(find(a), []).append(items[a])
        out = []
        for mem in groups.values():
            # windows in ascending order; a new part starts when the sums
            # would exceed the cap
            mem.sort(key=lambda it: (it[1], sorted(it[0])))
            part: List[int] = []
            for srcs, w, r in mem:
                trial = sorted(set(part) | set(r["roots"]))
                comp, _, _ = plan.closure(trial, L)
                self._moment_registry(comp)
                nsum = sum(1 for k in self.mom if k[0] == "s")
                if part and nsum > SLIDE_MAX_SUMS:
                    out.append(part)
                    part = list(r["roots"])
                else:
                    part = trial
            if part:
                out.append(part)
        res = []
        for roots in out:
            roots = sorted(set(roots))
            comp, vr, wr = plan.closure(roots, L)
            res.append({"roots": roots, "comp": comp, "vr": vr, "wr": wr})
        self.mom = {}
        return res + rest

    def _weight(self, comp: Set[int]) -> float:
        ops = self.ops
        w = 0.0
        for i in comp:
            k = ops[i]["k"]
            if k == "ForeachBackWindow":
                w += (ops[i]["window"] - ops[i].get("segment_end", 0)) * 4
            elif k == "SkipListState":
                w += ops[i]["window"] * 12
        return w

    def _par_roles(self, roots: List[int], L: int) -> List[dict]:
        """Independent parts of a parallel level (no shared computed op) run as
        separate kernels: each gets its own registers and time chunking.  Cheap
        pointwise parts are kept together."""
        plan = self.plan
        closures = []
        for r in roots:
            comp, vr, wr = plan.closure([r], L)
            closures.append(([r], comp, vr, wr))
        # union components that share computed ops (not constants)
        groups: List[list] = []
        for c in closures:
            merged = [c]
            rest = []
            for g in groups:
                gcomp = set().union(*[x[1] for x in g])
                shared = {i for i in (gcomp & c[1]) if self.ops[i]["k"] != "ConstantOp"}
                if shared:
                    merged += g
                else:
                    rest.append(g)
            groups = rest + [merged]
        heavy, light = [], []
        for g in groups:
            comp = set().union(*[x[1] for x in g])
            (heavy if self._weight(comp) >= 40 else light).append(g)
        parts = heavy + ([sum(light, [])] if light else [])
        out = []
        for g in parts:
            rts = sorted(sum([x[0] for x in g], []))
            comp, vr, wr = plan.closure(rts, L)
            out.append({"roots": rts, "comp": comp, "vr": vr, "wr": wr})
        return out

    def _mem_ptr(self, j: int, decl: List[str], seen: Set[int]):
        """Pointer b{j} + stride st{j} of op j's [T][S] series."""
        if j in seen:
            return
        seen.add(j)
        op = self.ops[j]
        T = self.T
        k = op["k"]
        if k in ("Input", "Output"):
            sl = self.slot(op["buf"])
            const = "const " if k == "Input" else ""
            lay = self.layout_of(op)
            user = self.is_user_input(op)
            rowoff = "start" if user else "0"
            rows = "total_time" if user else "length"
            if op.get("single_value"):
                decl.append(f"  {const}{T}* __restrict__ b{j} = ({const}{T}*)P.p[{sl}] + s;")
                decl.append(f"  const long long st{j} = 0;")
            elif lay == "TS":
                decl.append(f"  {const}{T}* __restrict__ b{j} = ({const}{T}*)P.p[{sl}] + {rowoff} * S + s;")
                decl.append(f"  const long long st{j} = S;")
            else:
                L = self.blocking
                decl.append(f"  {const}{T}* __restrict__ b{j} = ({const}{T}*)P.p[{sl}] + "
                            f"(s / {L}) * {rows} * {L} + {rowoff} * {L} + s % {L};")
                decl.append(f"  const long long st{j} = {L};")
        else:
            sc = self.scratch[j]
            decl.append(f"  {T}* __restrict__ b{j} = ({T}*)P.w[{sc}] + s;")
            decl.append(f"  const long long st{j} = S;")

    # ------------------------------------------------------------------ ops
    def emit_top(self, i: int, ind: str, loops: Dict, comp: Set[int]):
        ops, T = self.ops, self.T
        op = ops[i]
        k = op["k"]
        a = op["in"]
        fplan = self.fplan
        if k == "Input":
            return  # loaded at the top of the iteration
        if k in ("Output", "WindowedTempOutput"):
            self.lines.append(f"{ind}b{i}[t * st{i}] = {self.val(a[0])};")
            self.lines.append(f"{ind}const {T} v{i} = {self.val(a[0])};")
        elif k == "ForeachBackWindow":
            body, reds, own = loops[i]
            w, seg = op["window"], op.get("segment_end", 0)
            for r in own:
                self.lines.append(f"{ind}{self.reduction_decl(r)}")
            self.lines.append(f"{ind}for (int iter = {w - 1}; iter >= {seg}; --iter) {{")
            bind = ind + "  "
            for j in body:
                bo = ops[j]
                if bo["k"] == "IterValue":
                    self.lines.append(f"{bind}const {T} v{j} = {self.window_read(bo['in'][1], 'iter')};")
                elif bo["k"] == "WindowLoopIndex":
                    self.lines.append(f"{bind}const {T} v{j} = ({T})({bo.get('loop_window', w)} - 1 - iter);")
                elif not self.emit_simple(j, bind, fplan):
                    raise Unsupported(f"op in loop body: {bo['k']}")
            for r in reds:
                self.reduction_step(r, fplan, bind)
            self.lines.append(f"{ind}}}")
        elif k in REDUCTIONS:
            pass
        elif k == "BackRef":
            # in a time chunk a BackRef still reads the real earlier row
            rd = (StageGen.window_read(self, a[0], op['window']) if self.chunk_mode
                  else self.window_read(a[0], op['window']))
            self.lines.append(f"{ind}const {T} v{i} = {rd};")
        elif k == "FastWindowedSum" and self.slide:
            w = op["window"]
            nn, sm = self.mom[("nn", a[0], w)], self.mom[("s", ((a[0], 1),), w)]
            self.lines.append(f"{ind}const {T} v{i} = ({nn} == 0) ? ({T}){sm} : kun::knan<{T}>();")
        elif k == "SlideReduce":
            val = self._slide_value(i, ind)
            self.lines.append(f"{ind}const {T} v{i} = {val};")
        elif k == "FastWindowedSum":
            self.lines.append(f"{ind}const {T} v{i} = ({T})fw{i}.step({self.window_read(a[0], op['window'])}, {self.val(a[0])});")
        elif k == "WindowedLinearRegression":
            shared = "true" if contraction.regression_shares_square(ops, i) else "false"
            self.lines.append(f"{ind}lr{i}.template step<{shared}>({self.window_read(a[0], op['window'])}, {self.val(a[0])});")
        elif k == "WindowedLinearRegressionRSqaureImpl":
            self.lines.append(f"{ind}const {T} v{i} = ({T})lr{a[0]}.rsq();")
        elif k == "WindowedLinearRegressionSlopeImpl":
            self.lines.append(f"{ind}const {T} v{i} = ({T})lr{a[0]}.slope();")
        elif k == "WindowedLinearRegressionResiImpl":
            self.lines.append(f"{ind}const {T} v{i} = ({T})lr{a[0]}.resi({self.val(a[1])});")
        elif k == "ExpMovingAvg":
            self.lines.append(f"{ind}const {T} v{i} = ema{i}.step({self.val(a[0])});")
        elif k == "Accumulator":
            self.lines.append(f"{ind}const {T} v{i} = acc{i};")
        elif k == "SetAccumulator":
            acc = a[0]
            self.lines.append(f"{ind}acc{acc} = kun::ksel({self.val(a[1])}) ? {self.val(a[2])} : v{acc};")
            self.lines.append(f"{ind}const {T} v{i} = acc{acc};")
        elif k == "SkipListState":
            self.lines.append(f"{ind}sl{i}.step({self.val(a[0])}, {self.val(a[1])}, (int)t);")
        elif k in SL_CONS and self._reg_window(a[0]):
            if k == "SkipListQuantile":
                self.lines.append(f"{ind}const {T} v{i} = {self._quantile(i)};")
            elif k == "SkipListMin":
                self.lines.append(f"{ind}const {T} v{i} = sl{a[0]}.vmin();")
            elif k == "SkipListMax":
                self.lines.append(f"{ind}const {T} v{i} = sl{a[0]}.vmax();")
            elif k == "SkipListArgMin":
                self.lines.append(f"{ind}const {T} v{i} = sl{a[0]}.argmin(t);")
            else:
                self.lines.append(f"{ind}const {T} v{i} = sl{a[0]}.rank({self.val(a[1])});")
        elif k == "SkipListQuantile":
            self.lines.append(f"{ind}const {T} v{i} = sl{a[0]}.quantile<{T}>({self.lit(op['q'])});")
        elif k == "SkipListMin":
            self.lines.append(f"{ind}const {T} v{i} = sl{a[0]}.vmin<{T}>();")
        elif k == "SkipListMax":
            self.lines.append(f"{ind}const {T} v{i} = sl{a[0]}.vmax<{T}>();")
        elif k == "SkipListArgMin":
            self.lines.append(f"{ind}const {T} v{i} = sl{a[0]}.argmin<{T}>(t);")
        elif k == "SkipListRank":
            self.lines.append(f"{ind}const {T} v{i} = sl{a[0]}.rank<{T}>({self.val(a[1])});")
        elif not self.emit_simple(i, ind, fplan):
            raise Unsupported(f"op {k}")

    def _loops(self):
        ops = self.ops
        loops = {}
        prev = None
        n = len(ops)
        for i, op in enumerate(ops):
            if op["k"] != "ForeachBackWindow":
                continue
            body, reds = [], []
            if op.get("copy_prev_body") and prev is not None:
                body += loops[prev][0]
                reds += loops[prev][1]
            own = [j for j in range(n) if ops[j]["k"] in REDUCTIONS
                   and contraction.reduction_loop(ops, j) == i]
            body += [j for j in range(n) if ops[j].get("p", -1) == i]
            reds += own
            loops[i] = (body, reds, own)
            prev = i
        return loops

    def _state_decl(self, i: int) -> Optional[str]:
        op, T = self.ops[i], self.T
        k = op["k"]
        if k == "SlideReduce" or (k == "FastWindowedSum" and self.slide):
            return None  # window sums of the role's moment registry
        if k == "FastWindowedSum":
            return f"kun::FWSum<{self.RT}> fw{i}({op['window']});"
        if k == "Accumulator":
            return f"{T} acc{i} = 0;"
        if k == "WindowedLinearRegression":
            if self.slide:
                return f"kun::SlideLinReg<{op['window']}> lr{i};"
            return f"kun::LinReg<{self.RT}, {op['window']}> lr{i};"
        if k == "ExpMovingAvg":
            init = f"kun::knan<{T}>()"
            if len(op["in"]) == 2:
                init = f"b{op['in'][1]}[0]"
            return f"kun::EMA<{T}, {op['window']}> ema{i}({init});"
        if k == "SkipListState":
            if self._reg_window(i):
                idx = "true" if any(q["k"] == "SkipListArgMin" and q["in"][0] == i for q in self.ops) else "false"
                return f"kun::RegWindow<{T}, {op['window']}, {idx}> sl{i};"
            return f"kun::SortedWindow<{op['window']}> sl{i};"
        return None

    # ------------------------------------------------------------ moments
    def _moment_registry(self, comp: Set[int]):
        """Window sums and NaN counts the role's running sums need, each
        once: ("nn", series, w) counts the NaN rows of a series in the
        window; ("s", monomial, w) is the two-float window sum of a monomial
        (a product of series values of one row) over its rows whose factors
        are all numbers."""
        ops = self.ops
        mom: Dict[tuple, str] = {}

        def need(key):
            if key not in mom:
                mom[key] = (f"nn{len(mom)}" if key[0] == "nn" else f"sm{len(mom)}")

        for i in sorted(comp):
            op = ops[i]
            if op["k"] == "FastWindowedSum":
                need(("nn", op["in"][0], op["window"]))
                need(("s", ((op["in"][0], 1),), op["window"]))
            elif op["k"] == "SlideReduce":
                ns, w = op["nsrc"], op["window"]
                srcs = op["in"][:ns]
                for x in srcs:
                    need(("nn", x, w))
                for _, se, _ in op["terms"]:
                    mono = self._mono(srcs, se)
                    if mono:
                        need(("s", mono, w))
        self.mom = mom

    @staticmethod
    def _mono(srcs: List[int], exps: List[int]) -> tuple:
        d: Dict[int, int] = {}
        for x, e in zip(srcs, exps):
            if e:
                d[x] = d.get(x, 0) + e
        return tuple(sorted(d.items()))

    def _moment_decls(self, ind: str) -> List[str]:
        out = []
        for key, name in self.mom.items():
            if key[0] == "nn":
                out.append(f"{ind}int {name} = {key[2]};")
            else:
                out.append(f"{ind}kun::DFloat {name};")
        return out

    def _moment_updates(self, ind: str):
        """One row of every window sum of the role: the row leaving the
        window is taken out (when all its factors are numbers), the new row
        added; products are exact two-float products."""
        L, T = self.lines, self.T
        olds: Dict[tuple, str] = {}
        for key in self.mom:
            if key[0] == "nn":
                _, x, w = key
                o = f"o{x}_{w}"
                olds[(x, w)] = o
                L.append(f"{ind}const {T} {o} = {self.window_read(x, w)};")
        for key, name in self.mom.items():
            if key[0] == "nn":
                _, x, w = key
                L.append(f"{ind}{name} += (int)(v{x} != v{x}) - (int)({olds[(x, w)]} != {olds[(x, w)]});")
        for key, name in self.mom.items():
            if key[0] != "s":
                continue
            _, mono, w = key
            for which in ("old", "new"):
                vals = {x: (olds[(x, w)] if which == "old" else f"v{x}") for x, _ in mono}
                ok = " && ".join(f"{vals[x]} == {vals[x]}" for x, _ in mono)
                fac = [vals[x] for x, e in mono for _ in range(e)]
                if len(fac) == 1:
                    upd = f"kun::df_acc({name}, {'-' if which == 'old' else ''}{fac[0]});"
                else:
                    fn = "df_acc_prod_neg" if which == "old" else "df_acc_prod"
                    upd = f"kun::{fn}({name}, {fac[0]}, {fac[1]});"
                L.append(f"{ind}if ({ok}) {upd}")

    def _slide_value(self, i: int, ind: str) -> str:
        """The expanded window polynomial, evaluated in two-float arithmetic
        from the window sums and the invariants (each term a window sum
        scaled by the invariants and the coefficient, accumulated with
        TwoSum), rounded once; NaN while a row of the window has a NaN
        operand."""
        op, T = self.ops[i], self.T
        ns, w = op["nsrc"], op["window"]
        srcs, invs = op["in"][:ns], op["in"][ns:]
        acc = f"pa{i}"
        self.lines.append(f"{ind}kun::DFloat {acc};")
        for c, se, ie in op["terms"]:
            mono = self._mono(srcs, se)
            term = self.mom[("s", mono, w)] if mono else f"kun::DFloat({float(w)!r}f)"
            for x, e in zip(invs, ie):
                for _ in range(e):
                    term = f"kun::df_scale({term}, {self.val(x)})"
            if c != 1:
                term = f"kun::df_scale({term}, {float(c)!r}f)"
            self.lines.append(f"{ind}kun::df_acc_pair({acc}, {term});")
        ok = " && ".join(f"{self.mom[('nn', x, w)]} == 0" for x in sorted(set(srcs)))
        return f"(({ok}) ? ({T}){acc} : kun::knan<{T}>())"

    def _reg_window(self, i: int) -> bool:
        return self.ops[i]["window"] <= REG_WINDOW_MAX

    def _quantile(self, i: int) -> str:
        """SkipListQuantile with idx = int(q*(W-1)) and its fraction folded at
        generation time in the module dtype (Quantile.hpp:94-101)."""
        import numpy as np
        from .codegen import _f32_exact
        from fractions import Fraction
        op = self.ops[i]
        st = op["in"][0]
        W = self.ops[st]["window"]
        if self.dtype == "float":
            q = np.float32(_f32_exact(op["q"]))
            iwf = np.float32(q * np.float32(W - 1))
            idx = int(iwf)
            exact = np.float32(idx) == iwf
            frac = np.float32(iwf - np.float32(idx))
        else:
            q = float(Fraction(op["q"]))
            iwf = q * float(W - 1)
            idx = int(iwf)
            exact = float(idx) == iwf
            frac = iwf - float(idx)
        if exact:
            return f"sl{st}.template quantile<{idx}, true>(({self.T})0)"
        return f"sl{st}.template quantile<{idx}, false>({self.lit(repr(float(frac)))})"

    def _body(self, comp: Set[int], vr: Set[int], stores: List[int], loops, ind: str):
        ops, T = self.ops, self.T
        self.cur_comp = comp
        for j in sorted(vr):
            if ops[j]["k"] == "Input" and ops[j].get("single_value"):
                self.lines.append(f"{ind}const {T} v{j} = b{j}[0];")
            else:
                self.lines.append(f"{ind}const {T} v{j} = b{j}[t * st{j}];")
        for i in range(len(ops)):
            if i in comp and ops[i].get("p", -1) < 0:
                self.emit_top(i, ind, loops, comp)
        for i in stores:
            self.lines.append(f"{ind}b{i}[t * st{i}] = {self.val(i)};")

    def window_read(self, src: int, off) -> str:
        key = (src, str(off))
        if self.pf_window is not None and key in self.pf_window:
            return f"{self.pf_window[key]}[u]"
        return super().window_read(src, off)

    def _scan_block(self, role: dict) -> int:
        """Rows per prefetch block: fewer when the role reads many series, so
        the prefetched rows stay in registers."""
        ops = self.ops
        n = len(role["vr"]) + sum(1 for i in role["comp"]
                                  if ops[i]["k"] in ("FastWindowedSum", "WindowedLinearRegression", "BackRef"))
        n += sum(ops[i]["nsrc"] for i in role["comp"] if ops[i]["k"] == "SlideReduce")
        if self.slide:
            # chunked scans have threads enough to hide memory latency; keep
            # the registers for the window sums (single-buffered)
            return SLIDE_BLOCK
        return SCAN_BLOCK if n <= 6 else (8 if n <= 12 else 4)

    def _scan_prefetch(self, role: dict, B: int, ind: str, chunk: bool = False):
        """Scan role body: rows are processed in blocks of B; every series the
        role reads (values at t and fixed-offset windowed reads) is loaded for
        the whole block first, so the B sequential state updates never wait on
        memory."""
        ops, T = self.ops, self.T
        comp, vr = role["comp"], role["vr"]
        stores = [i for i in role["roots"] if i in self.mats]
        L = self.lines
        self.cur_comp = comp
        wins = {}
        for i in sorted(comp):
            k = ops[i]["k"]
            if k == "BackRef" and chunk:
                continue  # read directly: it sees rows before the chunk's warm-up
            if k in ("FastWindowedSum", "WindowedLinearRegression", "BackRef"):
                wins[(ops[i]["in"][0], str(ops[i]["window"]))] = f"pw{i}"
            elif k == "SlideReduce":
                for x in ops[i]["in"][:ops[i]["nsrc"]]:
                    wins.setdefault((x, str(ops[i]["window"])), f"pw{i}_{x}")
        # in a time chunk the scan runs rows [tw, t1) and stores [t0, t1); the
        # rows a state would take out before tw were never put in: NaN
        tbeg, tend, wlo = ("tw", "t1", "tw") if chunk else ("0LL", "length", "0")
        # double-buffered: the loads of block tb + B are issued before the
        # state updates of block tb, so memory latency overlaps the scan.
        # Regression roles compute long enough per row to hide the loads
        # and keep the registers instead (measured: 478 us single-buffered,
        # 608 us double-buffered at 2000 stocks)
        dbl = not any(ops[i]["k"] == "WindowedLinearRegression" for i in comp) and not self.slide
        series = [j for j in sorted(vr) if not (ops[j]["k"] == "Input" and ops[j].get("single_value"))]
        for j in sorted(vr):
            if j not in series:
                L.append(f"{ind}const {T} pv{j} = b{j}[0];")
        wnames = []
        for (src, off), name in wins.items():
            if name not in [w[2] for w in wnames]:
                wnames.append((src, off, name))

        def loads(pre: str, base: str, bi: str):
            for j in series:
                L.append(f"{bi}#pragma unroll")
                L.append(f"{bi}for (int u = 0; u < {B}; ++u) {pre}v{j}[u] = ({base} + u < {tend}) ? "
                         f"b{j}[({base} + u) * st{j}] : kun::knan<{T}>();")
            for src, off, name in wnames:
                L.append(f"{bi}#pragma unroll")
                L.append(f"{bi}for (int u = 0; u < {B}; ++u) {{ const long long r = {base} + u - {off}; "
                         f"{pre}{name[1:]}[u] = (r >= {wlo} && {base} + u < {tend}) ? b{src}[r * st{src}] : "
                         f"kun::knan<{T}>(); }}")

        if dbl:
            for j in series:
                L.append(f"{ind}{T} pv{j}[{B}], nv{j}[{B}];")
            for src, off, name in wnames:
                L.append(f"{ind}{T} {name}[{B}], n{name[1:]}[{B}];")
            loads("p", tbeg, ind)
        L.append(f"{ind}for (long long tb = {tbeg}; tb < {tend}; tb += {B}) {{")
        bi = ind + "  "
        if dbl:
            loads("n", f"(tb + {B})", bi)
        else:
            for j in series:
                L.append(f"{bi}{T} pv{j}[{B}];")
            for src, off, name in wnames:
                L.append(f"{bi}{T} {name}[{B}];")
            loads("p", "tb", bi)
        L.append(f"{bi}#pragma unroll")
        L.append(f"{bi}for (int u = 0; u < {B}; ++u) {{")
        bj = bi + "  "
        L.append(f"{bj}const long long t = tb + u;")
        L.append(f"{bj}if (t >= {tend}) break;")
        for j in sorted(vr):
            if ops[j]["k"] == "Input" and ops[j].get("single_value"):
                L.append(f"{bj}const {T} v{j} = pv{j};")
            else:
                L.append(f"{bj}const {T} v{j} = pv{j}[u];")
        self.pf_window = wins
        self.chunk_mode = chunk
        if self.slide:
            self._moment_updates(bj)
        if chunk:
            # warm-up rows only advance the states
            L.append(f"{bj}if (t < t0) {{")
            for i in sorted(comp):
                if ops[i]["k"] in ("WindowedLinearRegression", "FastWindowedSum") and ops[i].get("p", -1) < 0 \
                        and not (self.slide and ops[i]["k"] == "FastWindowedSum"):
                    self.emit_top(i, bj + "  ", {}, comp)
            L.append(f"{bj}  continue;")
            L.append(f"{bj}}}")
        loops = self._loops()
        for i in range(len(ops)):
            if i in comp and ops[i].get("p", -1) < 0:
                self.emit_top(i, bj, loops, comp)
        self.pf_window = None
        self.chunk_mode = False
        guard = ""
        for i in stores:
            L.append(f"{bj}{guard}b{i}[t * st{i}] = {self.val(i)};")
        L.append(f"{bi}}}")
        for j in series if dbl else []:
            L.append(f"{bi}#pragma unroll")
            L.append(f"{bi}for (int u = 0; u < {B}; ++u) pv{j}[u] = nv{j}[u];")
        for src, off, name in wnames if dbl else []:
            L.append(f"{bi}#pragma unroll")
            L.append(f"{bi}for (int u = 0; u < {B}; ++u) {name}[u] = n{name[1:]}[u];")
        L.append(f"{ind}}}")

    # ------------------------------------------------------------------ staged (TMA) form
    def _tma_eligible(self, comp: Set[int], vr: Set[int], wr: Set[int]) -> bool:
        """An elementwise kernel (no window reads) whose inputs are whole
        [T][S] series can stage its rows by bulk copies."""
        ops = self.ops
        if wr or not vr or len(vr) > 11:
            return False
        if any(ops[i]["k"] in ("BackRef", "ForeachBackWindow", "SkipListState") for i in comp):
            return False
        for j in vr:
            op = ops[j]
            if op.get("single_value"):
                return False
            if op["k"] in ("Input", "Output") and self.layout_of(op) != "TS":
                return False
        return True

    def _tma_kernel(self, kname: str, pstruct: str, ki: int, comp: Set[int], vr: Set[int], stores: List[int],
                    loops, decl: List[str], U: int) -> str:
        """The staged instance of an elementwise kernel: blocks of 128
        stocks; thread 0 copies kTmaRows rows of every input series into a
        shared-memory stage with cp.async.bulk (one copy per row: the
        block's stocks are contiguous), double-buffered on two mbarriers, and
        the block computes from the stage while the next one is in flight.
        Waits are bounded: on a time-out the kernel sets the error word and
        returns instead of hanging."""
        T = self.T
        series = sorted(vr)
        nin = len(series)
        self.tma_slot = {j: k for k, j in enumerate(series)}
        self.store_guard = "live && "
        saved = self.lines
        self.lines = []
        self._emit_par_vec(comp, vr, stores, loops, U, "        ")
        body = self.lines
        self.lines = saved
        self.tma_slot = None
        self.store_guard = ""
        self.tma_kernels[ki] = [self._series_base(j) for j in series]
        copies = "\n".join(
            f"        kun::bulk_copy_g2s(&kst_sm[{k}][b][r][0], (const char*)(b{j} - tid) + (tc + r) * st{j} * "
            f"(long long)sizeof({T}), rowb, &kst_bar[b]);" for k, j in enumerate(series))
        return f"""
__global__ void __launch_bounds__(128) {kname}_tma(const {pstruct} P) {{
  __shared__ __align__(128) {T} kst_sm[{nin}][2][kun::kTmaRows][128];
  __shared__ __align__(8) unsigned long long kst_bar[2];
  const int bx = blockIdx.x, by = blockIdx.y;
  const int tid = threadIdx.x;
  const long long S = P.S;
  const long long s = (long long)bx * 128 + tid;
  const bool live = s < S;
  const long long total_time = P.total_time, start = P.start, length = P.length;
  (void)total_time; (void)start;
{chr(10).join(decl)}
  const long long tile = P.tile[{ki}];
  const long long t0 = (long long)by * tile;
  const long long t1 = t0 + tile < length ? t0 + tile : length;
  const long long left = S - (long long)bx * 128;
  const uint32_t rowb = (uint32_t)((left < 128 ? left : 128) * (long long)sizeof({T}));
  const int nch = t1 > t0 ? (int)((t1 - t0 + kun::kTmaRows - 1) / kun::kTmaRows) : 0;
  if (tid == 0) {{
    kun::mbar_init(&kst_bar[0], 1);
    kun::mbar_init(&kst_bar[1], 1);
    kun::mbar_init_fence();
  }}
  __syncthreads();
  auto issue = [&](int c) {{
    const int b = c & 1;
    const long long tc = t0 + (long long)c * kun::kTmaRows;
    const int nr = (int)(t1 - tc < kun::kTmaRows ? t1 - tc : kun::kTmaRows);
    kun::fence_proxy_async_smem();
    kun::mbar_arrive_expect_tx(&kst_bar[b], (uint32_t)nr * {nin}u * rowb);
    for (int r = 0; r < nr; ++r) {{
{copies}
    }}
  }};
  if (tid == 0 && nch > 0) issue(0);
  for (int c = 0; c < nch; ++c) {{
    const int kb = c & 1;
    if (tid == 0 && c + 1 < nch) issue(c + 1);
    const bool got = kun::mbar_wait(&kst_bar[kb], (uint32_t)((c >> 1) & 1), kun::kTmaWaitLimit);
    if (!__syncthreads_and(got)) {{
      // copies that never completed: report, give those in flight a last
      // bounded wait (their stage must not be reused), and stop
      if (tid == 0) {{
        if (P.err) atomicExch(P.err, 1);
        kun::mbar_wait(&kst_bar[kb], (uint32_t)((c >> 1) & 1), kun::kTmaWaitLimit);
        if (c + 1 < nch) kun::mbar_wait(&kst_bar[kb ^ 1], (uint32_t)(((c + 1) >> 1) & 1), kun::kTmaWaitLimit);
      }}
      __syncthreads();
      return;
    }}
    const long long tc = t0 + (long long)c * kun::kTmaRows;
    for (long long t = tc; t < tc + kun::kTmaRows && t < t1; t += {U}) {{
{chr(10).join(body)}
    }}
    __syncthreads();
  }}
}}
"""

    def _series_base(self, j: int) -> str:
        """Host expression of series j's device base pointer in a launcher."""
        op = self.ops[j]
        if op["k"] in ("Input", "Output"):
            return f"P.p[{self.slot(op['buf'])}]"
        return f"P.w[{self.scratch[j]}]"

    # ------------------------------------------------------------------ vector form
    def _vload(self, j: int, texpr: str) -> str:
        """Read of series j at row `texpr`, NaN outside [0, length); the test
        is compiled out of the interior instance of the body (KE false).  In
        the staged instance the row comes from the shared-memory stage."""
        if self.tma_slot is not None:
            return (f"(live && ({texpr}) < t1) ? kst_sm[{self.tma_slot[j]}][kb][({texpr}) - tc][tid] "
                    f": kun::knan<{self.T}>()")
        self.edge_body = True
        return f"kun::ldw<KE>(b{j}, st{j}, (long long)({texpr}), length)"

    def _emit_par_vec(self, comp: Set[int], vr: Set[int], stores: List[int], loops, U: int, ind: str):
        ops, T = self.ops, self.T
        # a window queue holds the U rows in use and VEC_PREFETCH rows ahead
        QL = U + VEC_PREFETCH
        self.cur_comp = comp
        self.vec = True
        L = self.lines
        for j in sorted(vr):
            if ops[j]["k"] == "Input" and ops[j].get("single_value"):
                L.append(f"{ind}{T} v{j}[{U}]; for (int u = 0; u < {U}; ++u) v{j}[u] = b{j}[0];")
            else:
                L.append(f"{ind}{T} v{j}[{U}];")
                L.append(f"{ind}#pragma unroll")
                L.append(f"{ind}for (int u = 0; u < {U}; ++u) v{j}[u] = {self._vload(j, 't + u')};")
        queues: Dict[Tuple[int, int], str] = {}
        chain_head = {}
        for i in range(len(ops)):
            if ops[i]["k"] == "ForeachBackWindow":
                chain_head[i] = self.plan.loop_chain[i][0]
        fplan = self.fplan
        for i in range(len(ops)):
            if i not in comp or ops[i].get("p", -1) >= 0:
                continue
            op = ops[i]
            k = op["k"]
            a = op["in"]
            if k == "Input":
                continue
            if k in ("Output", "WindowedTempOutput"):
                L.append(f"{ind}{T} v{i}[{U}];")
                L.append(f"{ind}#pragma unroll")
                L.append(f"{ind}for (int u = 0; u < {U}; ++u) {{ v{i}[u] = {self.val(a[0])}; "
                         f"if ({self.store_guard}t + u < t1) b{i}[(t + u) * st{i}] = v{i}[u]; }}")
            elif k == "ForeachBackWindow" and self._ext_chain(self.plan.loop_chain[i], loops, U):
                if i == chain_head[i]:
                    self._emit_ext_chain(self.plan.loop_chain[i], loops, U, ind)
            elif k == "ForeachBackWindow":
                body, reds, own = loops[i]
                w, seg = op["window"], op.get("segment_end", 0)
                head = chain_head[i]
                for r in own:
                    rk = ops[r]["k"]
                    decl = self.reduction_decl(r)
                    if rk == "ReduceRank":
                        L.append(f"{ind}kun::RRank<{T}> r{r}[{U}];")
                        L.append(f"{ind}#pragma unroll")
                        L.append(f"{ind}for (int u = 0; u < {U}; ++u) r{r}[u].reset({self.val(ops[r]['in'][1])});")
                    else:
                        L.append(f"{ind}{decl.split(' r')[0]} r{r}[{U}];")
                srcs = sorted({ops[j]["in"][1] for j in body if ops[j]["k"] == "IterValue"})
                for src in srcs:
                    key = (head, src)
                    if key not in queues:
                        qn = f"q{head}_{src}"
                        queues[key] = qn
                        wh = ops[head]["window"]
                        L.append(f"{ind}{T} {qn}[{QL}];")
                        L.append(f"{ind}#pragma unroll")
                        L.append(f"{ind}for (int u = 0; u < {QL}; ++u) {qn}[u] = {self._vload(src, f't + u - {wh - 1}')};")
                L.append(f"{ind}#pragma unroll {VEC_UNROLL}")
                L.append(f"{ind}for (int iter = {w - 1}; iter >= {seg}; --iter) {{")
                bi = ind + "  "
                L.append(f"{bi}#pragma unroll")
                L.append(f"{bi}for (int u = 0; u < {U}; ++u) {{")
                bj = bi + "  "
                for j in body:
                    bo = ops[j]
                    if bo["k"] == "IterValue":
                        L.append(f"{bj}const {T} v{j} = {queues[(head, bo['in'][1])]}[u];")
                    elif bo["k"] == "WindowLoopIndex":
                        L.append(f"{bj}const {T} v{j} = ({T})({bo.get('loop_window', w)} - 1 - iter);")
                    else:
                        e = self.simple_expr(j, fplan)
                        if e is None:
                            raise Unsupported(f"op in loop body: {bo['k']}")
                        L.append(f"{bj}const {T} v{j} = {e};")
                for r in reds:
                    self._vstep(r, bj)
                L.append(f"{bi}}}")
                for src in srcs:
                    qn = queues[(head, src)]
                    L.append(f"{bi}#pragma unroll")
                    L.append(f"{bi}for (int u = 0; u < {QL - 1}; ++u) {qn}[u] = {qn}[u + 1];")
                    L.append(f"{bi}{qn}[{QL - 1}] = {self._vload(src, f't + {QL} - iter')};")
                L.append(f"{ind}}}")
            elif k in REDUCTIONS:
                pass
            elif k == "BackRef":
                L.append(f"{ind}{T} v{i}[{U}];")
                L.append(f"{ind}#pragma unroll")
                L.append(f"{ind}for (int u = 0; u < {U}; ++u) v{i}[u] = {self._vload(a[0], f't + u - {op['window']}')};")
            else:
                e = self.simple_expr(i, fplan)
                if e is None:
                    raise Unsupported(f"op {k} in a vector kernel")
                L.append(f"{ind}{T} v{i}[{U}];")
                L.append(f"{ind}#pragma unroll")
                L.append(f"{ind}for (int u = 0; u < {U}; ++u) v{i}[u] = {e};")
        for i in stores:
            L.append(f"{ind}#pragma unroll")
            L.append(f"{ind}for (int u = 0; u < {U}; ++u) if ({self.store_guard}t + u < t1) "
                     f"b{i}[(t + u) * st{i}] = {self.val(i)};")
        self.vec = False

    EXT_KINDS = {"ReduceMax": ("true", "false"), "ReduceMin": ("false", "false"),
                 "ReduceArgMax": ("true", "true"), "ReduceArgMin": ("false", "true")}

    def _ext_chain(self, chain: List[int], loops, U: int) -> bool:
        """A loop chain whose reductions are all Min/Max/ArgMin/ArgMax of a
        window value, over windows of at least U rows that all end at the
        row: the U rows of a step then share all but U-1 positions of each
        window (kun::RExt)."""
        ops = self.ops
        reds = loops[chain[-1]][1]
        if not reds or any(ops[r]["k"] not in self.EXT_KINDS for r in reds):
            return False
        if any(ops[ops[r]["in"][0]]["k"] != "IterValue" for r in reds):
            return False
        for a, b in zip(chain, chain[1:]):
            if ops[a].get("segment_end", 0) != ops[b]["window"]:
                return False
        if ops[chain[-1]].get("segment_end", 0) != 0:
            return False
        return all(ops[l]["window"] >= U for l in chain)

    def _emit_ext_chain(self, chain: List[int], loops, U: int, ind: str):
        """The U rows t..t+U-1 of a window of w rows: row u covers positions
        t+u-w+1 .. t+u.  Positions t+U-w .. t are common to all U rows and are
        stepped once (kun::RExt, longest window first, each window's state
        joining at its first position); each row then steps its older edge
        (t+u-w+1 .. t+U-1-w), continues with the common run and steps its
        newer edge (t+1 .. t+u).  In position order, as the loop would."""
        ops, T, L = self.ops, self.T, self.lines
        reds = loops[chain[-1]][1]
        win = {r: ops[contraction.reduction_loop(ops, r)]["window"] for r in reds}
        src = {r: ops[ops[r]["in"][0]]["in"][1] for r in reds}
        kind = {r: self.EXT_KINDS[ops[r]["k"]] for r in reds}

        def ext(r):
            mx, arg = kind[r]
            return f"kun::RExt<{T}, {mx}, {arg}>"

        for r in reds:
            L.append(f"{ind}kun::RVal<{T}> r{r}[{U}];")
        L.append(f"{ind}{{")
        bi = ind + "  "
        for r in reds:
            L.append(f"{bi}{ext(r)} c{r};")
        ws = sorted(set(win.values()), reverse=True)
        for n, w in enumerate(ws):
            hi, lo = w - U, (ws[n + 1] - U + 1 if n + 1 < len(ws) else 0)
            if hi < lo:
                continue
            active = [r for r in reds if win[r] >= w]
            L.append(f"{bi}#pragma unroll {VEC_UNROLL}")
            L.append(f"{bi}for (int d = {hi}; d >= {lo}; --d) {{")
            for s in sorted({src[r] for r in active}):
                L.append(f"{bi}  const {T} x{s} = {self._vload(s, 't - d')};")
            for r in active:
                L.append(f"{bi}  c{r}.step(x{src[r]}, ({T})(-d));")
            L.append(f"{bi}}}")
        # the edge rows: o{s}_{w}[k] = row t+1-w+k, n{s}[k] = row t+1+k (k < U-1)
        for s, w in sorted({(src[r], win[r]) for r in reds}):
            L.append(f"{bi}{T} o{s}_{w}[{U - 1}];")
            L.append(f"{bi}#pragma unroll")
            L.append(f"{bi}for (int k = 0; k < {U - 1}; ++k) o{s}_{w}[k] = {self._vload(s, f't + 1 - {w} + k')};")
        for s in sorted(set(src.values())):
            L.append(f"{bi}{T} n{s}[{U - 1}];")
            L.append(f"{bi}#pragma unroll")
            L.append(f"{bi}for (int k = 0; k < {U - 1}; ++k) n{s}[k] = {self._vload(s, 't + 1 + k')};")
        L.append(f"{bi}#pragma unroll")
        L.append(f"{bi}for (int u = 0; u < {U}; ++u) {{")
        bj = bi + "  "
        for r in reds:
            s, w = src[r], win[r]
            L.append(f"{bj}{{")
            L.append(f"{bj}  {ext(r)} a;")
            L.append(f"{bj}  #pragma unroll")
            L.append(f"{bj}  for (int k = u; k < {U - 1}; ++k) a.step(o{s}_{w}[k], ({T})(k + 1 - {w}));")
            L.append(f"{bj}  a.then(c{r});")
            L.append(f"{bj}  #pragma unroll")
            L.append(f"{bj}  for (int k = 0; k < u; ++k) a.step(n{s}[k], ({T})(k + 1));")
            res = f"a.arg(({T})u)" if kind[r][1] == "true" else "a.v"
            L.append(f"{bj}  r{r}[u].v = {res};")
            L.append(f"{bj}}}")
        L.append(f"{bi}}}")
        L.append(f"{ind}}}")

    def _vstep(self, r: int, ind: str):
        """Per-lane reduction step inside the lane loop."""
        ops = self.ops
        op = ops[r]
        k = op["k"]
        x = self.val(op["in"][0])
        if k == "ReduceAdd" and r in self.fplan:
            _, prod = self.fplan[r]
            po = ops[prod]
            A = self.val(po["in"][0])
            B = self.val(po["in"][1]) if po["k"] == "Mul" else self.lit(po["value"])
            loop = contraction.reduction_loop(ops, r)
            if contraction.loop_unrolled(ops, loop):
                first = ops[loop]["window"] - 1
                self.lines.append(f"{ind}if (iter == {first}) r{r}[u].step_fma_first({A}, {B}); "
                                  f"else r{r}[u].step_fma({A}, {B});")
            else:
                self.lines.append(f"{ind}r{r}[u].step_fma({A}, {B});")
        elif k in ("ReduceArgMax", "ReduceArgMin"):
            self.lines.append(f"{ind}r{r}[u].step({x}, iter);")
        else:
            self.lines.append(f"{ind}r{r}[u].step({x});")

    # ------------------------------------------------------------------ stage
    def gen_ts(self):
        ops, T = self.ops, self.T
        ks = self._kernels()
        loops = self._loops()
        # series read by a later kernel need a memory home
        for i, op in enumerate(ops):
            if op["k"] == "WindowedTempOutput" and op.get("p", -1) < 0:
                self.scratch[i] = len(self.scratch)
        reads = set()
        for kd in ks:
            groups = kd["roles"] if kd["kind"] in ("scan", "cscan") else [kd]
            for g in groups:
                reads |= g["vr"] | g["wr"]
        mats = sorted(j for j in reads if ops[j]["k"] not in ("Input", "Output", "WindowedTempOutput"))
        self.mats = set(mats)
        for j in mats:
            self.scratch[j] = len(self.scratch)
        srcs, calls, kinfo = [], [], []
        tma_src: List[str] = []
        knames = []
        pstruct = f"P_{self.kname}"
        for ki, kd in enumerate(ks):
            L = kd["level"]
            kname = f"{self.kname}_L{L}_{ki}"
            knames.append(kname)
            decl: List[str] = []
            seen: Set[int] = set()
            self.lines = []
            self.cur_level = L
            self.edge_body = False
            if kd["kind"] == "par":
                comp, vr, wr = kd["comp"], kd["vr"], kd["wr"]
                for j in sorted(vr | wr | {i for i in comp if ops[i]["k"] in ("Output", "WindowedTempOutput")}
                                | {i for i in comp if i in self.scratch}):
                    self._mem_ptr(j, decl, seen)
                for i in sorted(comp):
                    if ops[i]["k"] == "ExpMovingAvg" and len(ops[i]["in"]) == 2:
                        self._mem_ptr(ops[i]["in"][1], decl, seen)
                stores = [i for i in sorted(comp) if i in mats]
                sls = [i for i in sorted(comp) if ops[i]["k"] == "SkipListState"]
                states = [self._state_decl(i) for i in sls]
                wmax = max([ops[i]["window"] for i in sls] + [0])
                chunk = max(PAR_CHUNK, 4 * wmax)
                # the time tile is a launch parameter (tunable, a multiple of 4)
                self.lines.append(f"  const long long tile = P.tile[{ki}];")
                self.lines.append("  const long long t0 = (long long)by * tile;")
                self.lines.append("  const long long t1 = t0 + tile < length ? t0 + tile : length;")
                for sd in states:
                    self.lines.append(f"  {sd}")
                if sls:
                    # rebuild the order-statistic windows from the previous rows;
                    # only values inserted in this warm-up are removed
                    self.lines.append(f"  const long long tw = t0 > {wmax} ? t0 - {wmax} : 0;")
                    self.lines.append("  for (long long t = tw; t < t0; ++t) {")
                    for i in sls:
                        src = self.plan.windowed_source(i)
                        W = ops[i]["window"]
                        self.lines.append(f"    sl{i}.step((t - {W} >= tw) ? {self.read_at(src, f't - {W}')} : kun::knan<{T}>(), "
                                          f"{self.read_at(src, 't')}, (int)t);")
                    self.lines.append("  }")
                # wide kernels (many series in and out) keep one row per
                # iteration: the 4-row form would not fit in registers
                wide = len(vr) + len(stores) + sum(1 for i in comp if ops[i]["k"] == "Output") > WIDE_SERIES
                U = VEC_U if any(ops[i]["k"] == "ForeachBackWindow" for i in comp) else VEC_U_ELEM
                if sls or U <= 1 or wide:
                    self.lines.append("  for (long long t = t0; t < t1; ++t) {")
                    self._body(comp, vr, stores, loops, "    ")
                else:
                    self.lines.append(f"  for (long long t = t0; t < t1; t += {U}) {{")
                    self._emit_par_vec(comp, vr, stores, loops, U, "    ")
                    self.vec_u = U
                self.lines.append("  }")
                kinfo.append((chunk, 0))
                if not (sls or wide) and U == VEC_U_ELEM and self._tma_eligible(comp, vr, wr):
                    tma_src.append(self._tma_kernel(kname, pstruct, ki, comp, vr, stores, loops, decl, U))
            elif kd["kind"] == "cscan":
                # one scan role over a time tile of rows, after a warm-up of
                # its longest window; the tile is a launch parameter like a
                # time-parallel kernel's
                r = kd["roles"][0]
                rr = (r["vr"] | r["wr"] | {i for i in r["roots"] if i in self.scratch}
                      | {i for i in r["comp"] if ops[i]["k"] in ("Output", "WindowedTempOutput")})
                for j in sorted(rr):
                    self._mem_ptr(j, decl, seen)
                wmax = max(ops[i]["window"] for i in r["comp"] if ops[i]["k"] in FINITE_SEQ)
                self.lines.append(f"  const long long tile = P.tile[{ki}];")
                self.lines.append("  const long long t0 = (long long)by * tile;")
                self.lines.append("  const long long t1 = t0 + tile < length ? t0 + tile : length;")
                self.lines.append(f"  const long long tw = t0 > {wmax} ? t0 - {wmax} : 0;")
                for i in sorted(r["comp"]):
                    sd = self._state_decl(i)
                    if sd:
                        self.lines.append(f"  {sd}")
                self._moment_registry(r["comp"])
                self.lines += self._moment_decls("  ")
                self._scan_prefetch(r, self._scan_block(r), "  ", chunk=True)
                kinfo.append((max(64, (2 * wmax + 15) // 16 * 16), 0))
            else:
                roles = kd["roles"]
                self.lines.append("  switch (by) {")
                for ri, r in enumerate(roles):
                    self.lines.append(f"  case {ri}: {{")
                    # each role declares only the series it touches, so the
                    # roles do not share live pointer registers
                    rr = r["vr"] | r["wr"] | {i for i in r["roots"] if i in self.scratch}
                    for i in r["comp"]:
                        if ops[i]["k"] == "ExpMovingAvg" and len(ops[i]["in"]) == 2:
                            rr.add(ops[i]["in"][1])
                    rdecl: List[str] = []
                    for j in sorted(rr):
                        self._mem_ptr(j, rdecl, set())
                    self.lines += ["  " + x for x in rdecl]
                    for i in sorted(r["comp"]):
                        sd = self._state_decl(i)
                        if sd:
                            self.lines.append(f"    {sd}")
                    self._moment_registry(r["comp"])
                    self.lines += self._moment_decls("    ")
                    self._scan_prefetch(r, self._scan_block(r), "    ")
                    self.lines.append("  } break;")
                self.lines.append("  default: break;")
                self.lines.append("  }")
                kinfo.append((len(roles), 1))
            # the body takes its block coordinates as arguments, so the same
            # code serves a launch of one job and a grouped launch of many.
            # A vector-form body comes in two instances: KE (edge) tests every
            # row it reads against [0, length); the interior one serves tiles
            # whose reads, rows [t0 - wmax, t1 + fwd), all lie inside.
            if self.edge_body:
                wmax = max([int(o[k]) for o in ops for k in ("window", "loop_window")
                            if isinstance(o.get(k), int)] + [0]) + self.vec_u
                fwd = self.vec_u + VEC_PREFETCH
                tmpl = "template <bool KE> "
                pick = (f"  const long long t0_ = (long long)by * P.tile[{ki}];\n"
                        f"  const long long t1_ = t0_ + P.tile[{ki}] < P.length ? t0_ + P.tile[{ki}] : P.length;\n"
                        f"  if (t0_ >= {wmax} && t1_ + {fwd} <= P.length) {kname}_body<false>(P, bx, by);\n"
                        f"  else {kname}_body<true>(P, bx, by);")
            else:
                tmpl, pick = "", f"  {kname}_body(P, bx, by);"
            srcs.append(f"""
{tmpl}__device__ __forceinline__ void {kname}_body(const {pstruct}& P, const int bx, const int by) {{
  const long long S = P.S;
  const long long s = (long long)bx * blockDim.x + threadIdx.x;
  if (s >= S) return;
  const long long total_time = P.total_time, start = P.start, length = P.length;
  (void)total_time; (void)start;
{chr(10).join(decl)}
{chr(10).join(self.lines)}
}}
""")
            # time-parallel kernels also come compiled for 64 registers a
            # thread (8 blocks of 128 threads an SM), picked per kernel by the
            # tuner; scan kernels keep one instance
            for suf, minb in ([("", "KUN_TS_MINB"), ("_r", "8")] if kd["kind"] in ("par", "cscan")
                              else [("", "KUN_TS_MINB")]):
                srcs.append(f"""__global__ void __launch_bounds__(KUN_TS_THREADS, {minb}) {kname}{suf}(const {pstruct} P) {{
  const int bx = blockIdx.x, by = blockIdx.y;
{pick}
}}
__global__ void __launch_bounds__(KUN_TS_THREADS, {minb}) {kname}{suf}_grp(const {pstruct}* __restrict__ jobs, const kun::TileTable tt) {{
  const int j = kun::tile_job(tt, blockIdx.x);
  const {pstruct}& P = jobs[j];
  const int local = (int)blockIdx.x - tt.off[j];
  const int gx = (int)((P.S + blockDim.x - 1) / blockDim.x);
  const int bx = local % gx, by = local / gx;
{pick}
}}
""")
        nslots = max(1, len(self.slots))
        nscr = max(1, len(self.scratch))
        nk = len(ks)
        head = f"""
struct {pstruct} {{
  void* p[{nslots}];
  void* w[{nscr}];
  long long S, total_time, start, length;
  int tile[{nk}];
  int* err;
}};
"""
        self.kernel_info = [(d << 1) | sc for d, sc in kinfo]
        self.num_kernels_override = nk
        # per kernel: time tile (or roles) and block size, from the tuning
        # arrays when given
        sel = ["  P.err = a->error_flag;"]
        for k, (d, sc) in enumerate(kinfo):
            sel.append(f"  const int tb{k} = (a->tune_block && a->tune_block[{k}] > 0) ? a->tune_block[{k}] : KUN_TS_THREADS;")
            sel.append(f"  const int blk{k} = tb{k} & 0xffff;")
            if not sc:
                sel.append(f"  P.tile[{k}] = (a->tune_tile && a->tune_tile[{k}] > 0) ? a->tune_tile[{k}] : {d};")
            else:
                sel.append(f"  P.tile[{k}] = 0;")
        for k, (d, sc) in enumerate(kinfo):
            gy = str(d) if sc else f"(unsigned)((a->length + P.tile[{k}] - 1) / P.tile[{k}])"
            grid = f"dim3((unsigned)((a->num_stocks + blk{k} - 1) / blk{k}), {gy}), blk{k}, 0, (cudaStream_t)stream"
            if sc:
                calls.append(f"  {knames[k]}<<<{grid}>>>(P);")
            elif k in self.tma_kernels:
                # the staged instance: 128 threads, rows of whole 16-byte
                # units (S % 4 == 0) from 16-byte aligned series
                ok = " && ".join([f"kun::aligned16({e})" for e in self.tma_kernels[k]])
                calls.append(f"  if (kun::tma_enabled() && blk{k} == 128 && (a->num_stocks % 4) == 0 && {ok}) "
                             f"{knames[k]}_tma<<<{grid}>>>(P);\n"
                             f"  else if (tb{k} & KUN_BLOCK_REGCAP) {knames[k]}_r<<<{grid}>>>(P);\n"
                             f"  else {knames[k]}<<<{grid}>>>(P);")
            else:
                calls.append(f"  if (tb{k} & KUN_BLOCK_REGCAP) {knames[k]}_r<<<{grid}>>>(P);\n"
                             f"  else {knames[k]}<<<{grid}>>>(P);")
            calls.append("  if (cudaError_t e = cudaGetLastError()) return (int)e;")
        launch = self.launcher(pstruct, "\n".join(sel + calls))
        launch += self._group_launcher(pstruct, knames, kinfo)
        return head + "".join(srcs) + "".join(tma_src), launch

    def _group_launcher(self, pstruct: str, knames: List[str], kinfo) -> str:
        """prepare(): the parameter blocks of n jobs; launch_group(): every
        kernel of the stage once over all jobs' tiles."""
        fill = "\n".join(f"    P.p[{sl}] = a->buffers[{bid}];" for bid, sl in self.slots.items())
        fillw = "\n".join(f"    P.w[{sc}] = a->scratch[{sc}];" for sc in range(len(self.scratch)))
        tiles = []
        for k, (d, sc) in enumerate(kinfo):
            if sc:
                tiles.append(f"    P.tile[{k}] = 0;")
            else:
                tiles.append(f"    P.tile[{k}] = (a->tune_tile && a->tune_tile[{k}] > 0) ? a->tune_tile[{k}] : {d};")
        launches = []
        for k, (d, sc) in enumerate(kinfo):
            gy = str(d) if sc else f"(a->length + tile - 1) / tile"
            tl = "0" if sc else f"(a->tune_tile && a->tune_tile[{k}] > 0) ? a->tune_tile[{k}] : {d}"
            kcall = (f"{knames[k]}_grp<<<(unsigned)total, blk, 0, (cudaStream_t)stream>>>((const {pstruct}*)dev, tt);"
                     if sc else
                     f"if (tb & KUN_BLOCK_REGCAP) {knames[k]}_r_grp<<<(unsigned)total, blk, 0, (cudaStream_t)stream>>>"
                     f"((const {pstruct}*)dev, tt);\n      else {knames[k]}_grp<<<(unsigned)total, blk, 0, "
                     f"(cudaStream_t)stream>>>((const {pstruct}*)dev, tt);")
            launches.append(f"""  {{
    const int tb = (args[0].tune_block && args[0].tune_block[{k}] > 0) ? args[0].tune_block[{k}] : KUN_TS_THREADS;
    const int blk = tb & 0xffff;
    kun::TileTable tt;
    tt.njobs = njobs;
    long long total = 0;
    for (int j = 0; j < njobs; ++j) {{
      const KunGpuStageArgs* a = &args[j];
      const long long tile = {tl};
      (void)tile;
      tt.off[j] = (int)total;
      if (a->num_stocks > 0 && a->length > 0) total += ((a->num_stocks + blk - 1) / blk) * (long long)({gy});
    }}
    tt.off[njobs] = (int)total;
    if (total > 0x7fffffffLL) return (int)cudaErrorInvalidValue;
    if (total > 0) {{
      {kcall}
      if (cudaError_t e = cudaGetLastError()) return (int)e;
    }}
  }}""")
        return f"""
extern "C" size_t {self.kname}_prepare(const KunGpuStageArgs* args, int njobs, void* host) {{
  if (host) {{
    for (int j = 0; j < njobs; ++j) {{
      const KunGpuStageArgs* a = &args[j];
      {pstruct}& P = (({pstruct}*)host)[j];
{fill}
{fillw}
      P.S = a->num_stocks; P.total_time = a->total_time; P.start = a->start; P.length = a->length;
      P.err = a->error_flag;
{chr(10).join(tiles)}
    }}
  }}
  return sizeof({pstruct}) * (size_t)njobs;
}}

extern "C" int {self.kname}_launch_group(const KunGpuStageArgs* args, int njobs, const void* dev, void* stream) {{
  if (njobs <= 0) return 0;
  if (njobs > KUN_MAX_GROUP) return (int)cudaErrorInvalidValue;
{chr(10).join(launches)}
  return 0;
}}
"""
