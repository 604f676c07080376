// Drives the C++ mirror of the reference's simulator interface (include/CCUDAParticleSimulator.hpp)
// the way the reference's front end drives CBaseParticleSimulator: setupScene, then step() on
// a timer, reading the pass times and the state back. Exit code 0 = every check passed.
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "CCUDAParticleSimulator.hpp"

static int failures = 0;
#define CHECK(cond)                                                            \
    do {                                                                       \
        if (!(cond)) {                                                         \
            std::fprintf(stderr, "check failed: %s (line %d)\n", #cond, __LINE__); \
            failures++;                                                        \
        }                                                                      \
    } while (0)

int main(int argc, char **argv)
{
    const std::string logdir = argc > 1 ? argv[1] : ".";
    {
        CCUDAParticleSimulator sim(0.4f, DAM_BREAK);
        sim.setupScene();
        CHECK(sim.getParticlesCount() == 1620);  // the reference's assert, src/CBaseParticleSimulator.cpp:56
        CHECK(sim.getSelectedDevice().find("sm_") != std::string::npos);
        sim.start();
        for (int k = 0; k < 3; k++) sim.step();
        CHECK(sim.isRunning() && sim.getTotalIteration() == 3);
        const double *t = sim.lastPassTimes();
        CHECK(t[0] > 0 && t[1] > 0 && t[2] > 0 && t[3] == 0 && t[4] == 0);
        std::vector<float> xyz, vel, rho;
        sim.readState(xyz, vel, rho);
        bool finite = true;
        for (float v : xyz) finite = finite && std::isfinite(v);
        CHECK(finite);
        float rmin = 1e30f;
        for (float r : rho) rmin = r < rmin ? r : rmin;
        CHECK(rmin >= 328.0f);  // at least the self density m * poly6(0)
        const float g[3] = {1.0f, -9.80665f, 0.0f};
        sim.setGravityVector(g);
        sim.step();
        CHECK(sim.getTotalIteration() == 4);
        // the profiling log: events at iterations 0, 10, 20 and the reference's two CSV files
        for (int k = 0; k < 17; k++) sim.step();
        CHECK(sim.events.size() == 3 && sim.events[2].iteration == 20);
        CHECK(sim.events[1].updateForces > 0 && sim.events[2].fps > 0);
        // every pass returns its own time from its own call
        CHECK(sim.events[1].updateGrid > 0 && sim.events[1].updateDensityPressure > 0);
        CHECK(sim.exportLogs(logdir, "GPU CUDA", "Dam break"));
        FILE *f = std::fopen((logdir + "/Dam break_0.4.csv").c_str(), "r");
        CHECK(f != nullptr);
        if (f) {
            char line[512] = {0};
            CHECK(std::fgets(line, sizeof line, f) != nullptr);
            int semis = 0;
            for (char *q = line; *q; q++) semis += *q == ';';
            CHECK(std::string(line).rfind("GPU CUDA;", 0) == 0 && semis == 4);
            std::fclose(f);
        }
        // the handoff delivers the state of the moment it was queued while stepping goes on
        {
            std::vector<float> now_xyz, v0, r0;
            sim.readState(now_xyz, v0, r0);
            std::vector<float> handed(now_xyz.size(), -1.0f);
            sim.handoffPositions(handed.data());
            sim.step();
            sim.handoffWait();
            CHECK(handed == now_xyz);
        }
        sim.setOnlineTuning(4);
        for (int k = 0; k < 4; k++) sim.step();
        // an out-of-order pass makes the next step fail: the simulator stops and signals
        std::string msg;
        sim.errorOccured = [&](const char *m) { msg = m; };
        sim.updateGrid();
        sim.step();
        CHECK(!sim.isRunning() && !msg.empty());
    }
    {
        CCUDAParticleSimulator sim(0.4f, FOUNTAIN);
        sim.setupScene();
        CHECK(sim.getParticlesCount() == 0 && sim.getMaxParticlesCount() == 1620);
        for (int k = 0; k < 5; k++) sim.step();
        CHECK(sim.getParticlesCount() == 35);
    }
    std::printf("%s: %d failed checks\n", failures ? "FAIL" : "OK", failures);
    return failures ? 1 : 0;
}
