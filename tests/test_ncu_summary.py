"""libfalcon_dsp_gb300.ncu_summary: the ncu CSV fold the benchmark's
roofline.traffic is read from (profiles/*_dram.txt), on a synthetic capture:
ncu's own messages before the header, units other than bytes and ns,
thousands separators, templated kernel names, and the write/read round trip."""
from libfalcon_dsp_gb300 import ncu_summary as S

CSV = '''==PROF== Connected to process 1 (python)
some program output
"ID","Process ID","Process Name","Host Name","Kernel Name","Context","Stream","Block Size","Grid Size","Device","CC","Section Name","Metric Name","Metric Unit","Metric Value"
"0","1","python","h","void fdsp::tc_prep_kernel<0>(fdsp::TcLaunch, int)","1","13","(256, 1, 1)","(10, 1, 1)","0","10.3","Command line profiler metrics","dram__bytes_read.sum","Mbyte","2.5"
"0","1","python","h","void fdsp::tc_prep_kernel<0>(fdsp::TcLaunch, int)","1","13","(256, 1, 1)","(10, 1, 1)","0","10.3","Command line profiler metrics","dram__bytes_write.sum","byte","1,000,000"
"0","1","python","h","void fdsp::tc_prep_kernel<0>(fdsp::TcLaunch, int)","1","13","(256, 1, 1)","(10, 1, 1)","0","10.3","Command line profiler metrics","gpu__time_duration.sum","usecond","20"
"1","1","python","h","void fdsp::tc_filter_kernel<0>(fdsp::TcFilterParams)","1","13","(608, 1, 1)","(152, 1, 1)","0","10.3","Command line profiler metrics","dram__bytes_read.sum","Gbyte","1"
"1","1","python","h","void fdsp::tc_filter_kernel<0>(fdsp::TcFilterParams)","1","13","(608, 1, 1)","(152, 1, 1)","0","10.3","Command line profiler metrics","dram__bytes_write.sum","Gbyte","3"
"1","1","python","h","void fdsp::tc_filter_kernel<0>(fdsp::TcFilterParams)","1","13","(608, 1, 1)","(152, 1, 1)","0","10.3","Command line profiler metrics","gpu__time_duration.sum","msecond","2"
"2","1","python","h","void fdsp::tc_filter_kernel<0>(fdsp::TcFilterParams)","1","13","(608, 1, 1)","(152, 1, 1)","0","10.3","Command line profiler metrics","dram__bytes_read.sum","Gbyte","1"
"2","1","python","h","void fdsp::tc_filter_kernel<0>(fdsp::TcFilterParams)","1","13","(608, 1, 1)","(152, 1, 1)","0","10.3","Command line profiler metrics","dram__bytes_write.sum","Gbyte","1"
"2","1","python","h","void fdsp::tc_filter_kernel<0>(fdsp::TcFilterParams)","1","13","(608, 1, 1)","(152, 1, 1)","0","10.3","Command line profiler metrics","gpu__time_duration.sum","msecond","4"
'''


def test_fold_and_round_trip(tmp_path):
    p = tmp_path / "cap.csv"
    p.write_text(CSV)
    s = S.summarize(S.parse(str(p)), n_in=1_000_000, steps=1)
    assert set(s) == {"tc_prep_kernel", "tc_filter_kernel"}
    f = s["tc_filter_kernel"]
    assert f["launches"] == 2 and f["launches_per_step"] == 2
    assert f["dram_read_bytes_per_launch"] == 1e9 and f["dram_write_bytes_per_launch"] == 2e9
    assert f["ns_per_launch"] == 3e6
    assert f["dram_bytes_per_input_sample"] == 6000.0
    pr = s["tc_prep_kernel"]
    assert pr["dram_read_bytes_per_launch"] == 2.5e6 and pr["dram_write_bytes_per_launch"] == 1e6
    assert pr["ns_per_launch"] == 20000.0
    out = tmp_path / "x_dram.txt"
    S.write(s, str(out), 1_000_000, 1, "ncu ...", note="synthetic")
    d = S.read(str(out))
    assert d["tc_filter_kernel.dram_bytes_per_input_sample"] == 6000.0
    assert d["step.dram_bytes_per_input_sample"] == 6003.5
    assert d["n_in"] == 1_000_000 and d["command"] == "ncu ..."


def test_bench_reads_the_committed_traffic_summary():
    import importlib.util
    import os
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(root, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    t = bench.ncu_traffic("tc_filter_kernel_channelizer_256_dram", "tc_filter_kernel", 1 << 26)
    assert t is not None and t["source"].startswith("profiles/")
    # the filter bank moves more than the algorithmic 148.3 B per input
    # sample, but well under the 230.8 of the previous kernels
    assert 148.0 < t["bytes_per_input_sample"] < 230.0
    assert abs(t["bytes_per_step"] / (t["bytes_per_input_sample"] * (1 << 26)) - 1.0) < 1e-3
