"""The batched fusion's device work queue (k_fuse_queue), simulated on the
CPU: items (stage, scene, chunk) are numbered stage by stage, CTAs take item
numbers from one counter, and an item runs only once every item of its
scene's previous stage has finished.  Whatever order the CTAs start and run
in -- including CTAs that become resident late, and fewer CTAs than scenes
-- every schedule finishes: an item only waits for items with smaller
numbers, which running CTAs hold."""
import random


def plan(chunks):
    """chunks[k][v]: stage k's chunks for scene v -> the items in queue order."""
    items = []
    for k, per_scene in enumerate(chunks):
        for v, n in enumerate(per_scene):
            items += [(k, v)] * n
    return items


def simulate(chunks, ctas, seed, order=plan):
    rng = random.Random(seed)
    items = order(chunks)
    need = {(k, v): n for k, per in enumerate(chunks) for v, n in enumerate(per)}
    done = {key: 0 for key in need}
    nxt = 0
    held = {}                 # CTA -> item number it holds
    started = set()
    finished = 0
    for _ in range(100 * len(items) + 1000):
        if finished == len(items):
            return True
        # a CTA not yet resident may start at any time
        waiting_to_start = [c for c in range(ctas) if c not in started]
        if waiting_to_start and rng.random() < 0.3:
            started.add(rng.choice(waiting_to_start))
            continue
        if not started:
            continue
        c = rng.choice(sorted(started))
        if c not in held:
            if nxt >= len(items):
                continue
            held[c] = nxt
            nxt += 1
            continue
        k, v = items[held[c]]
        if k > 0 and done[(k - 1, v)] < need[(k - 1, v)]:
            continue  # waits (bounded in the kernel); another CTA runs
        done[(k, v)] += 1
        finished += 1
        del held[c]
    return False


def test_every_schedule_finishes():
    rng = random.Random(1)
    for trial in range(200):
        scenes = rng.randint(1, 9)
        stages = 5 + rng.choice([2, 4, 6])
        chunks = [[1] * scenes] + [[rng.randint(1, 6) for _ in range(scenes)] for _ in range(stages - 1)]
        ctas = rng.randint(1, 12)
        assert simulate(chunks, ctas, seed=trial), (trial, scenes, stages, ctas)


def test_dependency_order_is_what_the_kernel_waits_for():
    # stage k of a scene starts only after all of its stage k - 1 chunks
    chunks = [[1, 1], [3, 2], [2, 2]]
    items = plan(chunks)
    first = {}
    for i, key in enumerate(items):
        first.setdefault(key, i)
    for (k, v), i in first.items():
        if k > 0:
            assert all(j < i for j, key in enumerate(items) if key == (k - 1, v))


def test_the_simulation_sees_a_deadlock():
    # numbered the other way round (later stages first), one CTA takes a
    # stage-1 item and waits for a set-up item nobody can take
    reverse = lambda chunks: list(reversed(plan(chunks)))  # noqa: E731
    assert not simulate([[1, 1], [2, 2]], ctas=1, seed=0, order=reverse)
