"""Host logic of bench.py on CPU: clock summaries over the timed windows,
the peak and traffic figures it reads from committed files, and the
workload's image size against the library's layout rule."""
import bench
from spiralpir import params as P


def test_clock_summary_counts_only_timed_windows():
    c = bench.ClockSampler(0)
    # (time, sm MHz, max MHz, W, reasons): sw_power_cap at t=1, hw_slowdown at t=9
    c.samples = [(1.0, 2000.0, 2070.0, 500.0, 0x4), (2.0, 2070.0, 2070.0, 800.0, 0x0),
                 (3.0, 2070.0, 2070.0, 700.0, 0x1), (9.0, 900.0, 2070.0, 100.0, 0x8)]
    s = c.summary([(0.5, 3.5)])
    assert s["samples"] == 3 and s["sm_mhz"] == 2070.0 and s["sm_min_mhz"] == 2000.0
    assert s["power_w_max"] == 800.0 and s["reasons"] == ["sw_power_cap"]   # gpu_idle is not a reason
    assert s["timed_s"] == 3.0
    s = c.summary([(8.0, 10.0)])
    assert s["reasons"] == ["hw_slowdown"] and s["sm_mhz"] == 900.0
    assert c.summary([(20.0, 21.0)]) is None


def test_peaks_and_traffic_from_committed_files():
    peak, kind = bench.measured_peaks()
    assert kind in ("measured", "fallback") and peak > 1000
    tpeak, _ = bench.measured_peaks("bf16_tflops")
    assert tpeak > 100
    algo = 7_566_524_416
    traffic = bench.measured_traffic(algo)
    assert traffic is None or 0.95 * algo < traffic < 1.2 * algo


def test_workload_image_size_matches_layout():
    sh = P.SHAPE_1GIB
    assert P.PARAMS.db_device_bytes(sh.nu1, sh.nu2) == bench.WORKLOAD["db_device_bytes"] == 7 << 30
    # packed 28-bit residues: 7 bytes per plaintext coefficient
    assert P.PARAMS.db_device_bytes(sh.nu1, sh.nu2) == sh.num_records * P.PARAMS.T * P.D * 7


def test_cpu_oracle_small_shape_matches_itself_and_decodes():
    """The CPU leg on a small shape: a full answer, timed, decodes to the
    record; the multiply timer runs at a shape other than the database's."""
    from spiralpir import client as C

    p, sh = P.PARAMS, P.DbShape(7, 3)
    cl = C.Client(p, seed=5)
    keys = cl.public_keys(sh.nu1, sh.nu2)
    recs = C.random_records(sh, p, seed=6)
    orc = bench.CpuOracle(p, sh, recs, keys)
    resp, secs = orc.answer(cl.query(sh, 9))
    assert secs > 0 and (cl.decode(resp) == recs[9]).all()
    assert orc.db_mul_s(6, 2) > 0


def test_integer_roofline_from_the_committed_counts():
    """Items per batch and the issue-slot fractions that bench.py reports
    next to each batch (profiles/int_pipe.json)."""
    p, sh = P.PARAMS, P.SHAPE_1GIB
    assert bench.expansion_outputs(p, sh.nu1, sh.nu2) == 1142
    r = bench.int_roofline(p, sh, 32, {"fold": 7.11, "expand": 4.58}, 2070.0)
    if r is None:
        return
    assert r["fold"]["items"] == {"k_fold_level<1>": 32 * 4 * 255, "k_acc_to_raw": 32 * 4 * 2 * 256}
    assert sum(r["expand"]["items"].values()) == 32 * 1142
    for stage in ("fold", "expand"):
        assert 0.2 < r[stage]["issue_frac"] < 1.2 and 0.1 < r[stage]["alu_pipe_frac"] < 1.2


def test_expansion_outputs_by_kernel():
    """The library's kernel choice per round, as the bench counts it: one
    query runs no round on the paired kernel (its widest rounds have fewer
    than 4 x SMs parents); 32 queries run rounds 5-9 on it."""
    p, sh = P.PARAMS, P.SHAPE_1GIB
    per_round = bench.expansion_round_outputs(p, sh.nu1, sh.nu2)
    assert sum(per_round) == 1142 and len(per_round) == p.g(sh.nu1, sh.nu2)
    one = bench.expansion_kernel_outputs(p, sh.nu1, sh.nu2, 1)
    assert one == {"k_expand_round<1>": 1142, "k_expand_pair": 0}
    b32 = bench.expansion_kernel_outputs(p, sh.nu1, sh.nu2, 32)
    assert b32["k_expand_pair"] == 32 * sum(per_round[5:])
    assert b32["k_expand_round<1>"] == 32 * sum(per_round[:5])


class _FakeLib:
    """The calls bench.stage_split makes, recorded."""

    def __init__(self, fail_at=None):
        self.timing, self.log, self.runs, self.fail_at = False, [], 0, fail_at

    def set_stage_timing(self, on):
        self.timing = on
        self.log.append(("timing", on))

    def run_staged(self, count):
        self.runs += 1
        if self.runs == self.fail_at:
            raise RuntimeError("run failed")
        self.log.append(("run", count, self.timing))

    def stats_reset(self):
        self.log.append(("reset",))

    def stats(self):
        return {"ms_expand": 3.0, "ms_total": 6.0, "answers": 3, "db_mul_by_variant": [3, 0, 0]}


def test_stage_split_times_with_stage_timing_and_restores_it():
    """Two capture runs, then the timed runs, all with the library's stage
    timing on; the ms fields per run; the timing off again afterwards, also
    when a run fails."""
    g = _FakeLib()
    st = bench.stage_split(g, 4, runs=3)
    assert st["ms_expand"] == 1.0 and st["ms_total"] == 2.0
    assert st["answers"] == 3 and st["db_mul_by_variant"] == [3, 0, 0]
    assert g.log[0] == ("timing", True) and g.log[-1] == ("timing", False)
    assert g.log.index(("reset",)) == 3          # after the two capture runs
    assert all(e[2] for e in g.log if e[0] == "run") and g.runs == 5
    bad = _FakeLib(fail_at=4)
    try:
        bench.stage_split(bad, 2, runs=3)
    except RuntimeError:
        pass
    assert bad.timing is False
