"""The profiling log export restates MainWindow::exportLogs (src/mainwindow.cpp:310-368):
file names, separators, labels and number format. Host only."""
import os


def test_export_logs_format(sphlib, tmp_path):
    E = sphlib.ProfilingEvent
    events = [E(0, 0.0, 0.5, 1.25, 2.0, 0.0, 0.0), E(10, 61.5, 0.0625, 0.3, 0.700001, 0.0, 0.0),
              E(20, 60.0, 1e-05, 2.5e-06, 123456789.0, 0.0, 0.0)]
    assert events[1].together() == 0.0625 + 0.3 + 0.700001
    d = str(tmp_path / "logs")
    s, det = sphlib.export_logs(events, d, "Dam break", 0.4, "GPU CUDA")
    assert os.path.basename(s) == "Dam break_0.4.csv" and os.path.basename(det) == "Dam break_0.4_detail.csv"
    assert open(s).read() == "GPU CUDA;3.75;1.0625;1.23457e+08;\n"
    assert open(det).read() == ("GPU CUDA\n"
                                "Grid;0.5;0.0625;1e-05;\n"
                                "Density + pressure;1.25;0.3;2.5e-06;\n"
                                "Forces;2;0.700001;1.23457e+08;\n"
                                "Collisions;0;0;0;\n"
                                "Integrate;0;0;0;\n\n\n")
    # a second export appends, like the reference's QFile::Append
    sphlib.export_logs(events[:1], d, "Dam break", 0.4, "CPU")
    assert open(s).read().splitlines() == ["GPU CUDA;3.75;1.0625;1.23457e+08;", "CPU;3.75;"]
    # whole box sizes print without a decimal point (QString::number(1.0) == "1")
    s2, _ = sphlib.export_logs(events, d, "Fountain", 1.0, "GPU CUDA")
    assert os.path.basename(s2) == "Fountain_1.csv"
