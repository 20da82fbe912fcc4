// A host loop that keeps the particle state in pinned host memory, written
// against include/pica_gb300.hpp and the CUDA runtime: every step uploads the
// packed state range by range, pushes each range as soon as its upload is in,
// updates the fields, migrates, and downloads the state range by range again.
// Host copies run on copy streams of their own (copyStatePackedRange with a copy
// stream), the gather / scatter kernels on two more, and range r of step n+1
// goes up as soon as range r of step n is down.  The run is compared with the
// same steps taken without copies; prints "same" when particles and fields are
// equal bit for bit (FP32 cell form).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "pica_gb300.hpp"

using namespace pica_gb300;

#define CUDA_OK(call)                                                                 \
    do {                                                                              \
        cudaError_t e_ = (call);                                                      \
        if (e_ != cudaSuccess) {                                                      \
            std::printf("cuda error %s at line %d\n", cudaGetErrorString(e_), __LINE__); \
            std::exit(2);                                                             \
        }                                                                             \
    } while (0)

static Config makeConfig(double& n0, double& h) {
    n0 = 1e18;
    const double wp = std::sqrt(4 * constants::pi * n0 * constants::electronCharge * constants::electronCharge /
                                constants::electronMass);
    h = 0.05 * constants::c / wp;
    Config cfg;
    cfg.numCells = Int3(16, 8, 8);
    cfg.numCellsPerSupercell = Int3(4, 4, 4);
    cfg.step = FP3(h, h, h);
    cfg.dt = 0.5 * h / (constants::c * std::sqrt(3.0));
    cfg.form = Form::FP32Cell;
    cfg.shape = Shape::TSC;
    cfg.depositor = Depositor::Esirkepov;
    cfg.resortEvery = 2;
    return cfg;
}

static void fill(Simulation& sim, double n0, double h) {
    auto& ens = sim.ensemble();
    const Int3 n = sim.grid().getSize();
    for (int i = 0; i < n.x; i++)
        for (int j = 0; j < n.y; j++)
            for (int k = 0; k < n.z; k++)
                for (int p = 0; p < 6; p++) {
                    Particle3d q;
                    q.position = FP3((i + 0.1 + 0.15 * p) * h, (j + 0.9 - 0.13 * p) * h, (k + 0.2 + 0.11 * p) * h);
                    q.p = FP3(0.2 * std::sin(1.0 + i + 2 * p), 0.2 * std::cos(0.5 * j + p), 0.15 * std::sin(k - p));
                    q.factor = n0 * h * h * h / 6;
                    ens.add(q);
                }
    ens.upload();
    auto& grid = sim.grid();
    for (int i = 0; i < n.x; i++)
        for (int j = 0; j < n.y; j++)
            for (int k = 0; k < n.z; k++) {
                grid.ex(i, j, k) = 300.0 * std::sin(0.4 * i + j);
                grid.bz(i, j, k) = 200.0 * std::cos(0.3 * k - i);
            }
    grid.upload();
}

int main(int argc, char** argv) {
    const int steps = argc > 1 ? std::atoi(argv[1]) : 5;
    const int nr = argc > 2 ? std::atoi(argv[2]) : 4;
    const int comps = 8;   // FP32 cell form: cell, 3 offsets, 3 momenta, weight
    double n0, h;
    const Config cfg = makeConfig(n0, h);

    Simulation ref(cfg);
    fill(ref, n0, h);
    ref.step(steps);

    Simulation sim(cfg);
    fill(sim, n0, h);
    int lo, hi;
    CUDA_OK(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    cudaStream_t mainS, up, upc, down, downc;
    CUDA_OK(cudaStreamCreateWithFlags(&mainS, cudaStreamNonBlocking));
    for (cudaStream_t* s : {&up, &upc, &down, &downc}) CUDA_OK(cudaStreamCreateWithPriority(s, cudaStreamNonBlocking, hi));
    sim.setStream(mainS);

    const Int3 nsc = sim.ensemble().getNumSupercells();
    const int tot = nsc.x * nsc.y * nsc.z;
    std::vector<int32_t> bounds(nr + 1);
    for (int r = 0; r <= nr; r++) bounds[r] = (int32_t)((int64_t)tot * r / nr);

    int64_t slots = sim.statePackedSlots();
    const int64_t alloc = 2 * slots + 4096;   // room for the layout to grow
    std::vector<void*> host(comps);
    for (auto& p : host) CUDA_OK(cudaHostAlloc(&p, (size_t)alloc * 4, cudaHostAllocDefault));
    for (int c = 0; c < comps; c++) sim.copyStatePacked(0, c, host[c], false);
    CUDA_OK(cudaStreamSynchronize(mainS));

    std::vector<cudaEvent_t> upped(nr), downed(nr);
    for (auto* v : {&upped, &downed})
        for (auto& e : *v) CUDA_OK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    cudaEvent_t stepped;
    CUDA_OK(cudaEventCreateWithFlags(&stepped, cudaEventDisableTiming));
    YeeSolver solver;
    for (int s = 0; s < steps; s++) {
        sim.setStream(up);
        for (int r = 0; r < nr; r++) {
            if (s > 0) CUDA_OK(cudaStreamWaitEvent(upc, downed[r], 0));   // range r of the last step is down
            for (int c = 0; c < comps; c++) sim.copyStatePackedRange(0, c, host[c], true, bounds[r], bounds[r + 1], upc);
            CUDA_OK(cudaEventRecord(upped[r], up));
        }
        sim.setStream(mainS);
        sim.pushDepositRanges(bounds, std::vector<void*>(upped.begin(), upped.end()));
        solver.updateB(sim.grid(), 0.5 * cfg.dt);
        solver.updateE(sim.grid(), cfg.dt);
        solver.updateB(sim.grid(), 0.5 * cfg.dt);
        sim.ensemble().migrate();
        slots = sim.statePackedSlots();   // the image of the new layout
        if (slots > alloc) {
            std::printf("layout outgrew the host buffers\n");
            return 1;
        }
        CUDA_OK(cudaEventRecord(stepped, mainS));
        CUDA_OK(cudaStreamWaitEvent(down, stepped, 0));
        sim.setStream(down);
        for (int r = 0; r < nr; r++) {
            for (int c = 0; c < comps; c++) sim.copyStatePackedRange(0, c, host[c], false, bounds[r], bounds[r + 1], downc);
            CUDA_OK(cudaEventRecord(downed[r], downc));
        }
        sim.setStream(mainS);
    }
    CUDA_OK(cudaDeviceSynchronize());

    bool same = sim.stepCount() == ref.stepCount() && sim.ensemble().counts() == ref.ensemble().counts();
    const auto pa = sim.ensemble().particles(), pr = ref.ensemble().particles();
    same = same && pa.size() == pr.size();
    for (size_t i = 0; same && i < pa.size(); i++)
        same = pa[i].position.x == pr[i].position.x && pa[i].position.y == pr[i].position.y &&
               pa[i].position.z == pr[i].position.z && pa[i].p.x == pr[i].p.x && pa[i].p.y == pr[i].p.y &&
               pa[i].p.z == pr[i].p.z && pa[i].factor == pr[i].factor;
    sim.grid().download();
    ref.grid().download();
    const Int3 n = sim.grid().getSize();
    for (int i = 0; same && i < n.x; i++)
        for (int j = 0; same && j < n.y; j++)
            for (int k = 0; same && k < n.z; k++) {
                auto& a = sim.grid();
                auto& b = ref.grid();
                same = a.ex(i, j, k) == b.ex(i, j, k) && a.ey(i, j, k) == b.ey(i, j, k) && a.ez(i, j, k) == b.ez(i, j, k) &&
                       a.bx(i, j, k) == b.bx(i, j, k) && a.by(i, j, k) == b.by(i, j, k) && a.bz(i, j, k) == b.bz(i, j, k) &&
                       a.jx(i, j, k) == b.jx(i, j, k) && a.jy(i, j, k) == b.jy(i, j, k) && a.jz(i, j, k) == b.jz(i, j, k);
            }
    std::printf("%lld particles, %d ranges, %s\n", (long long)pa.size(), nr, same ? "same" : "differ");
    for (auto& e : upped) cudaEventDestroy(e);
    for (auto& e : downed) cudaEventDestroy(e);
    cudaEventDestroy(stepped);
    for (auto p : host) cudaFreeHost(p);
    return same ? 0 : 1;
}
