"""The library's launch and batching rules (gpu-pir_gb300/csrc/plan.h),
compiled on the CPU with a small driver: the expansion kernel of each
round (and the Python mirror of it that bench.py uses to count each
kernel's items), the split schedules of the narrow launches, the pack
kernel choice, and the serving loop's batch selection."""
import os
import shutil
import subprocess

import pytest

import bench
from spiralpir import params as P

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "gpu-pir_gb300", "csrc")

DRIVER = r"""
#include <cstdio>
#include <deque>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>
#include "plan.h"
using namespace sp;

// The serving loop's selection on a queue whose requests are all valid:
// indices (into the queue, oldest first) of the next batch.
static std::vector<int> select_batch(const std::vector<int> &dbs, int cap) {
    std::vector<int> out;
    if (dbs.empty()) return out;
    const BatchRule rule = batch_rule(dbs.size(), cap, dbs.front());
    for (int i = 0; i < (int)dbs.size() && (int)out.size() < cap; i++)
        if (rule.takes(dbs[i])) out.push_back(i);
    return out;
}

int main() {
    std::string line;
    while (std::getline(std::cin, line)) {
        std::istringstream in(line);
        std::string op;
        in >> op;
        if (op == "expand") {
            unsigned long long max_out, nq, sms; int force;
            in >> max_out >> nq >> sms >> force;
            std::printf("%d\n", expand_kernel(max_out, nq, sms, force));
        } else if (op == "split") {
            unsigned long long sms, items, cap; int shift;
            in >> sms >> items >> cap >> shift;
            std::printf("%d\n", shifted_split(split_rule(sms, items, cap), shift, (int)cap));
        } else if (op == "packrow") {
            int n, scratch; unsigned long long nq, sms, counters;
            in >> n >> nq >> sms >> scratch >> counters;
            std::printf("%d\n", pack_by_row(n, nq, sms, scratch != 0, counters) ? 1 : 0);
        } else if (op == "foldnarrow") {
            unsigned long long folds, sms;
            in >> folds >> sms;
            std::printf("%d\n", fold_narrow(folds, sms) ? 1 : 0);
        } else if (op == "batch") {
            int cap, db; std::vector<int> dbs;
            in >> cap;
            while (in >> db) dbs.push_back(db);
            for (int i : select_batch(dbs, cap)) std::printf("%d ", i);
            std::printf("\n");
        }
    }
    return 0;
}
"""


@pytest.fixture(scope="module")
def rules(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    d = tmp_path_factory.mktemp("plan")
    src, exe = d / "driver.cpp", d / "driver"
    src.write_text(DRIVER)
    subprocess.run([cxx, "-std=c++17", "-O1", "-I", CSRC, str(src), "-o", str(exe)], check=True)

    def run(lines):
        r = subprocess.run([str(exe)], input="\n".join(lines) + "\n", capture_output=True, text=True, check=True)
        return r.stdout.splitlines()
    return run


SPLIT, SINGLE, PAIR = 1, 2, 3


def test_expansion_kernel_per_round_matches_the_bench_counts(rules):
    """expand_kernel over every round of the 1 GiB workload agrees with the
    rule bench.py counts each kernel's items by (paired once a round has
    4 x SMs parents, split below 2 x SMs outputs)."""
    p, sh = P.PARAMS, P.SHAPE_1GIB
    g = p.g(sh.nu1, sh.nu2)
    per_round = bench.expansion_round_outputs(p, sh.nu1, sh.nu2)
    for B in (1, 2, 8, 16, 32, 64):
        got = [int(x) for x in rules([f"expand {2 << r} {B} 152 0" for r in range(g)])]
        paired = sum(B * per_round[r] for r in range(g) if got[r] == PAIR)
        counts = bench.expansion_kernel_outputs(p, sh.nu1, sh.nu2, B)
        assert counts["k_expand_pair"] == paired, B
        for r in range(g):
            outs = (2 << r) * B
            assert (got[r] == SPLIT) == (outs < 2 * 152), (B, r)
    # one query: the eight narrow rounds split, the two wide ones one CTA per output
    one = [int(x) for x in rules([f"expand {2 << r} 1 152 0" for r in range(g)])]
    assert one == [SPLIT] * 8 + [SINGLE] * 2
    # a forced kernel runs every round
    assert rules(["expand 2 1 152 3", "expand 1024 64 152 1", "expand 1024 64 152 2"]) == ["3", "1", "2"]


def test_split_schedules(rules):
    # rule min(SMs / items, cap), at least 1; shifts multiply or divide by
    # powers of two within [1, cap]; SPLIT_NONE gives 1
    cases = {
        "split 152 2 4 0": 4, "split 152 64 4 0": 2, "split 152 200 4 0": 1,
        "split 152 16 7 0": 7, "split 152 16 7 -1": 3, "split 152 16 7 -16": 1,
        "split 152 64 7 1": 4, "split 152 64 7 4": 7, "split 152 64 7 -4": 1,
        "split 152 6 9 0": 9, "split 152 20 9 -1": 3,
    }
    assert [int(x) for x in rules(list(cases))] == list(cases.values())


def test_pack_and_fold_kernel_choice(rules):
    got = rules([
        "packrow 2 1 152 1 4096",    # one query, n = 2: 6 polynomials, by row
        "packrow 2 25 152 1 4096",   # 150 <= 152
        "packrow 2 26 152 1 4096",   # 156 > 152: by column
        "packrow 4 7 152 1 4096",    # 140
        "packrow 4 8 152 1 4096",    # 160
        "packrow 2 1 152 0 4096",    # no split scratch (the pack stage entry)
        "packrow 1 76 152 1 4096",
        "packrow 1 77 152 1 4096",
        "foldnarrow 128 152", "foldnarrow 152 152", "foldnarrow 153 152",
    ])
    assert got == ["1", "1", "0", "1", "0", "0", "1", "0", "1", "1", "0"]


def test_serving_batch_selection(rules):
    """A queue that fits one batch runs whole in arrival order; a longer one
    takes the oldest request's database first, in arrival order, up to the
    lane's capacity, and leaves the other requests in place."""
    got = rules([
        "batch 4 1 2 1 3",                 # fits: all, in order
        "batch 4 1 2 1 3 1",               # 5 > 4: database 1 first
        "batch 2 2 1 2 1 2 2",             # database 2, first two of its requests
        "batch 3 7",                        # one request
        "batch 3",                          # empty queue
        "batch 3 5 5 5 5 5",               # one database, longer than a batch
    ])
    assert [list(map(int, g.split())) for g in got] == [
        [0, 1, 2, 3], [0, 2, 4], [0, 2], [0], [], [0, 1, 2]]
