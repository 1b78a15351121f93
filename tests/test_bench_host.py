"""Host-side pieces of bench.py (no GPU): the frozen work model, molecule
dimensions, padding, the workload description and the clock summary."""
import numpy as np
import pytest

import bench


def test_work_model_per_pass_and_precision_split():
    n = np.array([100.0, 200.0])
    k = np.array([45.0, 90.0])
    passes = np.array([10, 20])
    passes32 = np.array([6, 15])
    fl = bench.flop_model(n, k, passes, passes32)
    f64, f32 = fl["tridiag"]
    assert f64 == pytest.approx(4 / 3 * (4 * 100 ** 3 + 5 * 200 ** 3))
    assert f32 == pytest.approx(4 / 3 * (6 * 100 ** 3 + 15 * 200 ** 3))
    b64, _ = fl["backtransform"]
    assert b64 == pytest.approx(2 * (4 * 100 * 100 * 45 + 5 * 200 * 200 * 90))
    c64, c32 = fl["cholesky"]
    assert c32 == 0.0 and c64 == pytest.approx(sum((2 / 3 + 3) * x ** 3 for x in (100, 200)))


def test_molecule_dims_counts_aos_and_occupied_orbitals():
    h2o = (np.array([8, 1, 1]), np.zeros((3, 3)))
    ch4 = (np.array([6, 1, 1, 1, 1]), np.zeros((5, 3)))
    n, kocc = bench.molecule_dims([h2o, ch4])
    assert n.tolist() == [8, 12]       # O 2s2p + 2 x H 1s2s; C 2s2p + 4 x H 1s2s
    assert kocc.tolist() == [4.0, 4.0]  # 8 valence electrons each


def test_pad_and_workload_config():
    mols = [(np.array([1, 1]), np.ones((2, 3))), (np.array([8, 1, 1]), 2 * np.ones((3, 3)))]
    num, pos = bench.pad(mols)
    assert num.shape == (2, 3) and pos.shape == (2, 3, 3)
    assert num[0].tolist() == [1, 1, 0] and np.all(pos[0, 2] == 0)
    cfg = bench.workload_config(4, 512)
    assert cfg["global_batch"] == 2048 and cfg["molecules_per_gpu"] == 512
    assert "molecule shards" in cfg["parallelism"]


def test_clock_summary_parses_nvidia_smi_rows(tmp_path):
    clk = bench.ClockSampler(0)
    rows = ["0, 2070, 2070, 900.5, 0x0, Not Active, Not Active, Not Active, Not Active",
            "0, 1980, 2070, 1300.0, 0x4, Not Active, Not Active, Not Active, Active",
            "0, 2070, 2070, 1000.0, 0x0, Not Active, Not Active, Not Active, Not Active"]
    with open(clk.file.name, "w") as f:
        f.write("\n".join(rows) + "\n")
    s = clk.summary()
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"] and s["samples"] == 3


def test_size_matched_sample_spans_the_size_range():
    mols = [(np.ones(n, dtype=int), None) for n in [50, 10, 120, 30, 70, 90, 11, 119]]
    idx = bench.size_matched(mols, 4)
    sizes = [len(mols[i][0]) for i in idx]
    assert sizes == sorted(sizes) and sizes[0] == 10 and sizes[-1] == 120
    assert len(set(idx)) == 4


def test_parity_summary_classifies_every_molecule():
    class R:
        pass

    import torch

    r = R()
    r.energy = torch.tensor([1.0, 2.0 + 5e-9, 3.5, 4.0 + 1e-6, 5.0, 6.0])
    r.status = np.array([0, 0, 0, 0, 1, 0])
    r.iterations = np.array([10, 11, 12, 13, 301, 14])
    r.fp32_passes = np.zeros(6, dtype=int)
    ref = {"energy": np.array([1.0, 2.0, 3.0, 4.0, 5.0, 6.0]),
           "converged": np.array([True, True, True, True, True, False]),
           "iterations": np.array([10, 12, 12, 13, 20, 301])}
    p = bench.parity_summary(r, ref, seconds=2.0)
    assert p["verified"] == 2 and p["other_state"] == 1 and p["imprecise"] == 1
    assert p["reference_only_converged"] == 1 and p["both_converged"] == 4
    assert p["verified_rate"] == 1.0 and p["iterations_equal_to_reference"] == 1
