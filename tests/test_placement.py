"""Device placement of the three splits, checked on the host (corrx_plan_query).

The checks are those the reference's multi_device.c makes on a live context
(corr-cuda/tests/multi_device.c:84-212 and its check_plan_shape): time slice and
baseline range give every device every station in order; the range split tiles
the baseline axis contiguously; pair covering gives each device a proper,
sorted subset, every baseline to exactly one device holding both stations, and
resident sets that differ by at most one station. On top of those: each
reported baseline's local index names the same (j, k) pair in the device's own
numbering, which is what the fetch's gather relies on.
"""

from __future__ import annotations

import itertools

import pytest

SPLITS = {"range": 0, "covering": 1, "time_slice": 2}


def pairs(n):
    return [(j, k) for j in range(n) for k in range(j, n)]


def query_all(pkg, n, nd, split):
    cfg = pkg.make_config(n, 2048, 32, 32, 2, 1, split_mode=split, devices=list(range(nd)))
    return [pkg.plan_query(cfg, d) for d in range(nd)]


def check_plan(n, nd, split, plans):
    """Raise AssertionError when a placement breaks a rule of its split."""
    nb = n * (n + 1) // 2
    allp = pairs(n)
    owner = {}
    nxt = 0
    for d, p in enumerate(plans):
        st, bl, lo = p["stations"], p["baselines"], p["local"]
        assert p["device_id"] == d
        assert p["n_baseline"] == len(bl) > 0
        assert p["n_station_resident"] == len(st)
        assert st == sorted(set(st)) and all(0 <= s < n for s in st)
        assert p["first_baseline"] == bl[0]
        assert p["contiguous"] == (bl == list(range(bl[0], bl[0] + len(bl))))
        lp = pairs(len(st))
        for b, l in zip(bl, lo):
            j, k = allp[b]
            lj, lk = lp[l]
            assert (st[lj], st[lk]) == (j, k), "local index names another pair"
        if split in (SPLITS["range"], SPLITS["time_slice"]):
            assert st == list(range(n))
        if split == SPLITS["time_slice"]:
            assert bl == list(range(nb))
        else:
            for b in bl:
                assert b not in owner, f"baseline {b} owned twice"
                owner[b] = d
        if split == SPLITS["range"]:
            assert p["contiguous"] and bl[0] == nxt
            nxt += len(bl)
    if split != SPLITS["time_slice"]:
        assert sorted(owner) == list(range(nb)), "a baseline is owned by no device"
    if split == SPLITS["covering"]:
        sizes = [len(p["stations"]) for p in plans]
        assert max(sizes) - min(sizes) <= 1
        if nd >= 3 and n >= 3:   # two stations can only be covered by holding both
            assert max(sizes) < n, "a device holds every station: nothing is covered"


@pytest.mark.parametrize("split", list(SPLITS.values()), ids=list(SPLITS))
@pytest.mark.parametrize("nd", range(1, 9))
def test_every_split_follows_its_rules(pkg, split, nd):
    for n in (1, 2, 3, 4, 8, 15, 24, 40, 44):
        if split != SPLITS["time_slice"] and nd > n * (n + 1) // 2:
            with pytest.raises(pkg.CorrError):   # some device would own nothing
                query_all(pkg, n, nd, split)
            continue
        check_plan(n, nd, split, query_all(pkg, n, nd, split))


def test_covering_residency_at_the_design_sizes(pkg):
    # two of three groups per device at 4 devices; half the array at 6
    assert [p["n_station_resident"] for p in query_all(pkg, 24, 4, 1)] == [16, 16, 16, 16]
    assert [p["n_station_resident"] for p in query_all(pkg, 24, 6, 1)] == [12] * 6
    res40 = [p["n_station_resident"] for p in query_all(pkg, 40, 4, 1)]
    assert max(res40) - min(res40) <= 1 and max(res40) <= 27
    # devices 1 and 2 alone hold group 2: its 36 inner pairs plus 64 cross pairs
    # each put at least 82 baselines there; the rest balance around that
    bl = [p["n_baseline"] for p in query_all(pkg, 24, 4, 1)]
    assert sum(bl) == 300 and max(bl) <= 84


def test_too_many_devices_is_refused(pkg):
    lib = pkg.abi.load()
    for split in SPLITS.values():
        if split == SPLITS["time_slice"]:
            continue
        cfg = pkg.make_config(2, 2048, 32, 32, 2, 1, split_mode=split, devices=list(range(4)))
        with pytest.raises(pkg.CorrError) as e:
            pkg.plan_query(cfg, 0)
        assert e.value.status == 1 and "no baselines" in e.value.message
    assert lib.corr_last_error()


def test_query_argument_errors(pkg):
    import ctypes as C
    lib = pkg.abi.load()
    cfg = pkg.make_config(4, 2048, 32, 32, 2, 1, split_mode=2, devices=[0, 1])
    plan = pkg.abi.corr_device_plan()
    assert lib.corrx_plan_query(C.byref(cfg), 2, C.byref(plan), None, 0, None, 0, None, 0) == 1
    short = (C.c_int32 * 3)()
    assert lib.corrx_plan_query(C.byref(cfg), 0, C.byref(plan), short, 3, None, 0, None, 0) == 1
    assert lib.corrx_plan_query(C.byref(cfg), 0, C.byref(plan), None, 0, None, 0, None, 0) == 0
    assert plan.n_baseline == 10 and plan.n_station_resident == 4
    cfg.struct_size = 4
    assert lib.corrx_plan_query(C.byref(cfg), 0, C.byref(plan), None, 0, None, 0, None, 0) == 2


def test_checker_catches_planted_mistakes(pkg):
    """Each planted error in a good plan must be caught by check_plan."""
    good = query_all(pkg, 8, 4, SPLITS["covering"])
    check_plan(8, 4, SPLITS["covering"], good)

    def broken(edit):
        plans = [dict(p, stations=list(p["stations"]), baselines=list(p["baselines"]),
                      local=list(p["local"])) for p in good]
        edit(plans)
        return plans

    def drop(ps):          # a baseline owned by nobody
        ps[0]["baselines"].pop()
        ps[0]["local"].pop()
        ps[0]["n_baseline"] -= 1

    def dup(ps):           # a baseline owned twice
        ps[1]["baselines"].append(ps[0]["baselines"][0])
        ps[1]["local"].append(ps[1]["local"][0])
        ps[1]["n_baseline"] += 1

    def wrong_local(ps):   # gather index pointing at another pair
        ps[2]["local"][0], ps[2]["local"][1] = ps[2]["local"][1], ps[2]["local"][0]

    def unbalanced(ps):    # resident sets two stations apart
        ps[3]["stations"] = ps[3]["stations"][:-2]
        ps[3]["n_station_resident"] -= 2

    for edit in (drop, dup, wrong_local, unbalanced):
        with pytest.raises(AssertionError):
            check_plan(8, 4, SPLITS["covering"], broken(edit))
    rng_plans = query_all(pkg, 8, 3, SPLITS["range"])
    rng_plans[1], rng_plans[2] = rng_plans[2], rng_plans[1]
    for d, p in enumerate(rng_plans):
        p["device_id"] = d
    with pytest.raises(AssertionError):   # ranges out of order
        check_plan(8, 3, SPLITS["range"], rng_plans)


@pytest.mark.parametrize("n,nd,split,ok", [
    (44, 1, "range", True),            # 990 baselines on one device
    (45, 1, "range", False),           # 1035 > 1024 on one device
    (45, 2, "range", True),            # 518 + 517
    (45, 2, "time_slice", False),      # every device owns every baseline
    (64, 3, "covering", True),         # about 2080 / 3 each
    (90, 4, "range", True),            # 4095 baselines: 1024, 1024, 1024, 1023
    (91, 4, "range", False),           # 4186: 1047 on a device
    (127, 8, "range", True),           # 8128: 1016 each
    (128, 8, "range", False),          # 8256: 1032 each
])
def test_per_device_baseline_limit(pkg, n, nd, split, ok):
    """The reference's limit is per device (corr-cuda/src/kernels.cu:474-483): at
    most 1024 baselines owned by any device, so more than 44 stations need their
    baselines split over several devices."""
    cfg = pkg.make_config(n, 2048, 32, 32, 2, 1, split_mode=SPLITS[split],
                          devices=list(range(nd)))
    if ok:
        plans = [pkg.plan_query(cfg, d) for d in range(nd)]
        assert max(p["n_baseline"] for p in plans) <= 1024
        check_plan(n, nd, SPLITS[split], plans)
    else:
        with pytest.raises(pkg.abi.CorrError) as e:
            pkg.plan_query(cfg, 0)
        assert e.value.status == pkg.abi.CORR_ERR_ARG
        assert "per device" in e.value.message


def test_station_limit(pkg):
    cfg = pkg.make_config(129, 2048, 32, 32, 2, 1, split_mode=SPLITS["range"],
                          devices=list(range(8)))
    with pytest.raises(pkg.abi.CorrError) as e:
        pkg.plan_query(cfg, 0)
    assert "128" in e.value.message
