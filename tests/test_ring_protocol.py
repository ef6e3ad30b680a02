"""CPU model of the shared-memory ring that streams the large color steps
of the single-launch ILU apply (k_ilu_coop, ring_produce / ring_wait_slice
in fpga_gb300/csrc/gbilu_kernels.cuh).

Lane st of the producer warp fills stage st with the CTA's slices
g = st (mod ns), in order, each after the compute warp that held slice
g - ns released the stage (the lanes run independently of each other; a
fill is a bulk copy whose bytes land later, in any order relative to other
copies); compute warp w takes the slices g = w (mod warps) of each large
step, and all compute warps meet at a barrier between steps while the
producer runs ahead into the next one. mbarrier parity waits are modelled
exactly: a wait on parity p returns at once when the barrier's current
phase parity differs from p, which is only right when the waiter is at most
one phase ahead.

The model checks, over random interleavings, stage counts, warp counts and
step sizes, that every compute warp reads the stage holding its own slice
and that every run ends; and that the protocol without the per-stage
sequence word (a warp waiting on the fill parity alone) reads stale stages
when there are fewer stages than compute warps -- the fault of a first
version of the ring on the GPU.
"""
import random


class Bar:
    """An mbarrier: expected arrivals per phase, transaction bytes, phase."""

    def __init__(self, count):
        self.count = count
        self.pending = count
        self.tx = 0
        self.phase = 0

    def arrive(self, tx=0):
        self.tx += tx
        self.pending -= 1
        self._advance()

    def complete_tx(self, nbytes):
        self.tx -= nbytes
        self._advance()

    def _advance(self):
        if self.pending == 0 and self.tx == 0:
            self.phase += 1
            self.pending = self.count

    def try_wait(self, parity):
        return (self.phase & 1) != parity


def run(ns, ncw, steps_sizes, seed, use_seq=True):
    rng = random.Random(seed)
    full = [Bar(1) for _ in range(ns)]
    empty = [Bar(1) for _ in range(ns)]
    seq = [-1] * ns          # slice number the producer last issued into a stage
    content = [None] * ns    # slice whose bytes have landed in a stage
    total = sum(steps_sizes)
    steps, base = [], 0
    for n in steps_sizes:
        steps.append(list(range(base, base + n)))
        base += n
    inflight = []
    issued = [0] * ns        # fills issued by each producer lane (one per stage)
    step = 0
    pos = [0] * ncw
    at_barrier = set()
    consumed = set()
    for _ in range(10 ** 6):
        if step == len(steps):
            break
        actors = [w for w in range(ncw) if w not in at_barrier]
        actors += [("lane", st) for st in range(ns) if st + issued[st] * ns < total]
        if inflight:
            actors.append("landing")
        a = rng.choice(actors)
        if isinstance(a, tuple):
            st = a[1]
            rnd = issued[st]
            g = st + rnd * ns
            if rnd > 0 and not empty[st].try_wait((rnd - 1) & 1):
                continue
            seq[st] = g
            full[st].arrive(tx=1)
            inflight.append((st, g))
            issued[st] += 1
        elif a == "landing":
            st, g = inflight.pop(rng.randrange(len(inflight)))
            content[st] = g
            full[st].complete_tx(1)
        else:
            mine = [g for g in steps[step] if g % ncw == a]
            if pos[a] >= len(mine):
                at_barrier.add(a)
                if len(at_barrier) == ncw:
                    at_barrier.clear()
                    step += 1
                    pos = [0] * ncw
                continue
            g = mine[pos[a]]
            st, rnd = g % ns, g // ns
            if use_seq and seq[st] != g:
                continue
            if not full[st].try_wait(rnd & 1):
                continue
            if content[st] != g:
                return False          # read a stale stage
            consumed.add(g)
            empty[st].arrive()
            pos[a] += 1
    assert step == len(steps) and len(consumed) == total, "the run did not end"
    return True


def test_ring_protocol_reads_its_own_slice_and_ends():
    for seed in range(1500):
        r = random.Random(seed)
        ns, ncw = r.randint(4, 16), r.randint(1, 15)
        sizes = [r.randint(0, 60) for _ in range(r.randint(1, 3))]
        assert run(ns, ncw, sizes, seed), (ns, ncw, sizes, seed)


def test_parity_only_waits_read_stale_stages():
    stale = sum(not run(7, 15, [60, 60], seed, use_seq=False) for seed in range(50))
    assert stale > 0
