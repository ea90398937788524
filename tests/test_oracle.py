"""CPU tests of the oracle: the reference's own unit tests restated, the grid
validator's tests, and the parity-tool semantics (no GPU)."""
from __future__ import annotations

import os
import subprocess

import numpy as np
import pytest


def bird(pos, vel, radius=0.0, next_decision=0.0):
    w = np.zeros(15, dtype=np.float32)
    w[0:3] = pos
    w[3:6] = vel
    w[8] = radius
    w[12] = next_decision
    return w


# ---- crates/flock-ref/src/state.rs:242-262 ----------------------------------
def test_file_round_trips(oracle, native, tmp_path):
    w = oracle.scatter(50, 7)
    w[3, 13] = np.uint32(9).view(np.float32)
    p = str(tmp_path / "a.flk")
    native.write_flk(p, 1.25, w)
    t, back = native.read_flk(p)
    assert t == 1.25
    assert back.tobytes() == w.tobytes()
    assert native.neighbours(back)[3] == 9


def test_scatter_is_repeatable_and_at_density(oracle):
    a = oracle.scatter(1000, 1)
    b = oracle.scatter(1000, 1)
    assert a.tobytes() == b.tobytes()
    side = np.cbrt(np.float32(1000.0) / np.float32(0.5))
    assert np.all(np.abs(a[:, 0]) <= side / 2)
    speed = np.linalg.norm(a[:, 3:6].astype(np.float64), axis=1)
    assert np.all(np.abs(speed - 10.0) < 1e-3)


# ---- crates/flock-ref/src/model.rs:208-269 ----------------------------------
def test_level_cruise_holds_height_and_speed(oracle):
    w = bird((0, 0, 100), (10, 0, 0))[None]
    for _ in range(200):
        w = oracle.integrate_all(w, threads=1)
    assert abs(w[0, 2] - 100.0) < 1.0, w[0, 2]
    assert abs(np.linalg.norm(w[0, 3:6]) - 10.0) < 0.5


def test_a_lone_bird_gets_only_roost_and_speed_forces(oracle):
    w = bird((0, 0, 100), (10, 0, 0), radius=1.5)[None]
    sets, dec = oracle.decide_many(w, np.array([0]))
    assert dec[0, 4].view(np.uint32) == 0
    assert np.linalg.norm(dec[0, 0:3]) < 1e-6


def test_two_close_birds_separate(oracle):
    w = np.stack([bird((0, 0, 100), (10, 0, 0), 2.0), bird((0, 0.5, 100), (10, 0, 0), 2.0)])
    sets, dec = oracle.decide_many(w, np.array([0]))
    assert dec[0, 4].view(np.uint32) == 1
    assert dec[0, 1] < 0.0, dec[0]


def test_settled_flock_neighbour_count_is_near_n_c(oracle):
    w = oracle.scatter(2000, 1)
    _, w = oracle.steps(w, 0.0, 200)
    mean = np.float32(oracle.stats(w)[1])
    assert abs(mean - 6.5) < 2.0, mean


# ---- cutile/src/main.rs:364-393 (check_grid) --------------------------------
def test_check_grid_accepts_a_correct_grid(oracle):
    assert oracle.check_grid([2, 0, 3, 3, 0], [0, 2, 2, 3, 5], [1, 4, 0, 2, 3], 4) == 0


def test_check_grid_rejects_a_wrong_total(oracle):
    assert oracle.check_grid([2, 0, 3, 3, 0], [0, 2, 2, 3, 4], [1, 4, 0, 2, 3], 4) == 3


def test_check_grid_rejects_a_bird_in_the_wrong_range(oracle):
    assert oracle.check_grid([2, 0, 3, 3, 0], [0, 2, 2, 3, 5], [1, 4, 2, 0, 3], 4) == 7


def test_check_grid_rejects_an_unstable_order(oracle):
    assert oracle.check_grid([2, 0, 3, 3, 0], [0, 2, 2, 3, 5], [4, 1, 0, 2, 3], 4) == 8


# ---- grid restatement (cuda/flock.cu:75-83, 368-372) ------------------------
@pytest.mark.parametrize("n", [0, 1, 2000, 100_000])
def test_oracle_grid_is_valid(oracle, n):
    w = oracle.scatter(n, 1)
    b = oracle.buckets_for(n)
    keys, offs, srt = oracle.grid(w, b)
    assert oracle.check_grid(keys, offs, srt, b, w) == 0
    # keys from the hash written out in numpy (flock.cu:77-83)
    c = np.floor(w[:, :3] * np.float32(0.25)).astype(np.int64).astype(np.uint32)
    h = (c[:, 0] * np.uint32(73856093)) ^ (c[:, 1] * np.uint32(19349663)) ^ (c[:, 2] * np.uint32(83492791))
    assert np.array_equal(keys, h & np.uint32(b - 1))


def test_buckets_for_matches_the_reference_rule(oracle):
    # next power of two >= 2n, clamped to [2^16, 2^22]
    for n, want in [(0, 1 << 16), (1000, 1 << 16), (32768, 1 << 16), (32769, 1 << 17), (100_000, 1 << 18),
                    (1_000_000, 1 << 21), (16_777_216, 1 << 22), (30_000_000, 1 << 22)]:
        assert oracle.buckets_for(n) == want


# ---- diff / statdiff semantics (main.rs:104-208) ----------------------------
def test_diff_and_statdiff_semantics(oracle):
    a = oracle.scatter(500, 3)
    ok, out, mm, ol = oracle.diff(a, a)
    assert ok and mm == 0 and ol == 0 and out.max() == 0
    b = a.copy()
    b[10, 0] += 2e-3  # one bird off by 2e-3 in x
    assert not oracle.diff(b, a)[0]
    ok, out, mm, ol = oracle.diff(b, a, allow=2, outlier_max=1e-2)
    assert ok and ol == 1
    c = a.copy()
    c[11, 13] = np.uint32(5).view(np.float32)  # a neighbour-count mismatch always fails
    assert not oracle.diff(c, a, allow=2)[0]
    assert oracle.statdiff(a, a)[0]
    d = a.copy()
    d[:, 8] += 0.02  # mean radius off by 0.02 > 0.01
    assert not oracle.statdiff(d, a)[0]


def test_oracle_cli_matches_the_reference_tool(oracle, tmp_path):
    g = str(tmp_path / "g.flk")
    s = str(tmp_path / "s.flk")
    assert subprocess.run([oracle.CLI, "gen", "--birds", "300", "--seed", "4", "--out", g]).returncode == 0
    assert subprocess.run([oracle.CLI, "step", "--in", g, "--steps", "3", "--out", s]).returncode == 0
    r = subprocess.run([oracle.CLI, "diff", s, s], capture_output=True, text=True)
    assert r.returncode == 0 and "PASS" in r.stdout and "neighbour-count mismatches 0 of 300" in r.stdout
    r = subprocess.run([oracle.CLI, "diff", g, s], capture_output=True, text=True)
    assert r.returncode == 1 and "FAIL" in r.stdout
    assert subprocess.run([oracle.CLI, "bogus"], capture_output=True).returncode == 2
    w = oracle.scatter(300, 4)
    t, back = oracle.steps(w, 0.0, 3)
    from murmuration_kernels_gb300 import read_flk

    t2, w2 = read_flk(s)
    assert t2 == np.float32(t) and w2.tobytes() == back.tobytes()


def test_step_sets_match_decide(oracle):
    w = oracle.scatter(1500, 2)
    t, after, sets, due = oracle.step(w, 0.0)
    idx = np.nonzero(due)[0]
    assert 0 < len(idx) < len(w)
    s2, dec = oracle.decide_many(w, idx)
    assert np.array_equal(sets[idx], s2)
    assert np.all(sets[~due] == 0)
    assert np.array_equal(after[idx, 9:12], dec[:, 0:3])
    nb = after[idx, 13].view(np.uint32)
    assert np.array_equal(nb, dec[:, 4].view(np.uint32))
    assert np.array_equal(sets[idx, 0], nb)


def test_fp64_twin_is_close(oracle):
    w = oracle.scatter(2000, 1)
    t, a, _, _ = oracle.step(w, 0.0)
    d = oracle.step_f64(w, 0.0)
    rel = np.abs(a[:, 0:6].astype(np.float64) - d[:, 0:6]) / np.maximum(np.abs(d[:, 0:6]), 1.0)
    assert rel.max() < 1e-5


def test_oracle_threads_do_not_change_results(oracle):
    w = oracle.scatter(3000, 5)
    _, a = oracle.steps(w, 0.0, 5, threads=1)
    _, b = oracle.steps(w, 0.0, 5, threads=0)
    assert a.tobytes() == b.tobytes()


def test_radius_step_matches_params_rs(oracle):
    # params.rs:61-65: r*(N_C/max(n,1))^(0.1/3) clamped to [R_H, R_MAX]
    assert oracle.radius_step(1.5, 0) == oracle.radius_step(1.5, 1)
    assert oracle.radius_step(150.0, 1) == np.float32(100.0)
    assert oracle.radius_step(0.1, 10_000) == np.float32(0.2)
    r = oracle.radius_step(1.5, 6)
    assert 1.5 < r < 1.51


def test_cpu_grid_step_matches_the_brute_force_oracle(oracle):
    # The CPU grid baseline (the reference GPU backend's cell walks on host
    # cores) decides like the brute-force oracle: same neighbour counts, radii
    # and next decisions; sums in another order agree to rounding.
    for n, seed, k in [(2000, 1, 3), (20_000, 4, 1)]:
        w = oracle.scatter(n, seed)
        tg, g = 0.0, w
        tc, c = 0.0, w
        for _ in range(k):
            tg, g = oracle.step_grid(g, tg)
            tc, c, _, _ = oracle.step(c, tc, with_sets=False)
        assert np.float32(tg) == np.float32(tc)
        ok, maxes, mism, _ = oracle.diff(g, c)
        assert ok and mism == 0, maxes
        assert np.array_equal(g[:, 8], c[:, 8]) and np.array_equal(g[:, 12], c[:, 12])
