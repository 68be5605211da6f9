// Drives the C++ plugin shims the way the reference's rendering view does
// (PhotonRenderingView.cpp:45-84): an animated OscCUDAMeshNode is collected
// into a GeometryList, a TriangleMap is built from it and the three tracers
// trace one frame.  Writes everything the test needs to compare with the
// oracle to the file named by argv[1]:
//   int32 T, int32 n, float tris[T*9], float o[n*3], float d[n*3],
//   then for restart, short-stack, brute: int32 hit[n], float t[n],
//   then float n0/n1/n2[T*4], uint8 c0[T*4] (the GeometryList attributes),
//   then for restart, short-stack, brute: uint8 rgba[n*4] (shaded Trace),
//   then for restart, short-stack, brute and 4 pixels each: HostTrace's
//   int32 hit, float t, uint8 rgba[4].
#include <cstdio>
#include <vector>

#include "kdgb_plugin.hpp"

using namespace OpenEngine;
using namespace OpenEngine::Scene;
using namespace OpenEngine::Utils::CUDA;

int main(int argc, char **argv)
{
    if (argc < 2) return 2;
    OscCUDAMeshNode osc(2.0f, 2.0f, 0.0f, 48);
    osc.Init();
    osc.Handle(350000);  // half a second of animation time

    const float model[16] = {1, 0, 0, 0.5f, 0, 1, 0, 0.25f, 0, 0, 1, 0.5f, 0, 0, 0, 1};
    GeometryList geom;
    geom.AddMesh(osc, model);

    TriangleMap map(&geom);
    // The SPLIT method is refused at Create(), as the reference's is.
    map.SetSplitMethod(TriangleMap::SPLIT);
    bool threw = false;
    try {
        map.Create();
    } catch (const Core::Exception &) {
        threw = true;
    }
    if (!threw) return 3;
    map.SetSplitMethod(TriangleMap::BOX);
    map.SetLowerAlgorithm(TriangleMap::SAH);
    map.Create();
    if (map.GetNodes()->GetSize() < 3) return 4;

    // An orthographic bundle of rays looking down -y at the field.
    const int side = 64, n = side * side;
    std::vector<float> o(3 * n), d(3 * n);
    for (int j = 0; j < side; ++j)
        for (int i = 0; i < side; ++i) {
            const int k = i + j * side;
            o[3 * k] = -0.45f + 1.9f * (i + 0.5f) / side;
            o[3 * k + 1] = 2.0f;
            o[3 * k + 2] = -0.45f + 1.9f * (j + 0.5f) / side;
            d[3 * k] = 0.01f;
            d[3 * k + 1] = -1.0f;
            d[3 * k + 2] = 0.02f;
        }
    float *od, *dd, *t, *u, *v;
    int *hit;
    cudaMalloc(&od, 12 * n);
    cudaMalloc(&dd, 12 * n);
    cudaMalloc(&t, 4 * n);
    cudaMalloc(&u, 4 * n);
    cudaMalloc(&v, 4 * n);
    cudaMalloc(&hit, 4 * n);
    cudaMemcpy(od, o.data(), 12 * n, cudaMemcpyHostToDevice);
    cudaMemcpy(dd, d.data(), 12 * n, cudaMemcpyHostToDevice);

    const int T = geom.GetSize();
    std::vector<float> tris(9 * (size_t)T);
    cudaMemcpy(tris.data(), geom.GetTriangleData(), tris.size() * 4, cudaMemcpyDeviceToHost);

    FILE *f = std::fopen(argv[1], "wb");
    if (!f) return 5;
    std::fwrite(&T, 4, 1, f);
    std::fwrite(&n, 4, 1, f);
    std::fwrite(tris.data(), 4, tris.size(), f);
    std::fwrite(o.data(), 4, o.size(), f);
    std::fwrite(d.data(), 4, d.size(), f);

    RayTracer restart(&map);
    ShortStack shortstack(&map);
    BruteTracer brute(&geom);
    IRayTracer *tracers[3] = {&restart, &shortstack, &brute};
    std::vector<int> h(n);
    std::vector<float> th(n);
    for (IRayTracer *tr : tracers) {
        tr->Trace(od, dd, n, hit, t, u, v);
        cudaMemcpy(h.data(), hit, 4 * n, cudaMemcpyDeviceToHost);
        cudaMemcpy(th.data(), t, 4 * n, cudaMemcpyDeviceToHost);
        std::fwrite(h.data(), 4, n, f);
        std::fwrite(th.data(), 4, n, f);
    }
    std::vector<float> nrm(4 * (size_t)T);
    for (const float *src : {geom.GetNormal0Data(), geom.GetNormal1Data(), geom.GetNormal2Data()}) {
        cudaMemcpy(nrm.data(), src, nrm.size() * 4, cudaMemcpyDeviceToHost);
        std::fwrite(nrm.data(), 4, nrm.size(), f);
    }
    std::vector<unsigned char> bytes(4 * (size_t)T);
    cudaMemcpy(bytes.data(), geom.GetColor0Data(), bytes.size(), cudaMemcpyDeviceToHost);
    std::fwrite(bytes.data(), 1, bytes.size(), f);
    uchar4 *canvas;
    cudaMalloc(&canvas, 4 * n);
    std::vector<unsigned char> px(4 * (size_t)n);
    for (IRayTracer *tr : tracers) {
        tr->Trace(od, dd, n, canvas);
        cudaMemcpy(px.data(), canvas, px.size(), cudaMemcpyDeviceToHost);
        std::fwrite(px.data(), 1, px.size(), f);
    }
    // HostTrace of pixels of the last traced image (side x side), after
    // one more shaded Trace per tracer so that each has rays to look up.
    const int probes[4][2] = {{0, 0}, {side / 2, side / 3}, {side - 1, 17}, {5, side - 1}};
    for (IRayTracer *tr : tracers) {
        tr->SetScreenWidth(side);
        tr->Trace(od, dd, n, canvas);
        for (const auto &xy : probes) {
            const HostTraceResult r = tr->HostTrace(xy[0], xy[1], tr == &brute ? nullptr : map.GetNodes());
            std::fwrite(&r.hit, 4, 1, f);
            std::fwrite(&r.t, 4, 1, f);
            std::fwrite(&r.color, 4, 1, f);
        }
        bool outside = false;
        try {
            tr->HostTrace(side, 0);
        } catch (const Core::Exception &) {
            outside = true;
        }
        if (!outside) return 6;
    }
    std::fclose(f);
    std::printf("plugin demo: %d triangles, %d nodes, build %.3f ms\n", T, map.GetNodes()->GetSize(),
                map.GetConstructionTime());
    return 0;
}
