// kdgb_plugin.hpp -- C++ plugin shims with the reference's class names over
// the C ABI in kdgb.h.
//
// OpenEngineDK/extensions-PhotonMapping calls its kd-tree path through these
// classes (Scene/KDNode.h, Scene/TriangleNode.h, Scene/CUDAMeshNode.h,
// Scene/OscCUDAMeshNode.h, Utils/CUDA/GeometryList.h, Utils/CUDA/TriangleMap.h,
// Utils/CUDA/IRayTracer.h and the three tracers).  The shims keep the names,
// the getters' meaning (raw device pointers, valid until the next rebuild) and
// the error behaviour (Core::Exception on failure); the scene graph, the
// OpenGL canvas and CUDADataBlock are not reproduced: meshes are added to the
// GeometryList explicitly and Trace writes first-hit buffers.
//
// Header only; link with -lkdgb -lcudart.
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "kdgb.h"

namespace OpenEngine {

namespace Core {
// Core::Exception of the reference (thrown on every failed call).
struct Exception : std::runtime_error {
    using std::runtime_error::runtime_error;
};
}  // namespace Core

namespace detail {
inline void check(int status, const char *where)
{
    if (status != KDGB_OK)
        throw Core::Exception(std::string(where) + ": " + kdgb_status_string(status) + " (" + kdgb_last_error() + ")");
}
inline void cuda(cudaError_t e, const char *where)
{
    if (e != cudaSuccess) throw Core::Exception(std::string(where) + ": " + cudaGetErrorString(e));
}
template <class T>
struct DeviceBuffer {
    T *p = nullptr;
    size_t n = 0;
    DeviceBuffer() = default;
    DeviceBuffer(const DeviceBuffer &) = delete;
    DeviceBuffer &operator=(const DeviceBuffer &) = delete;
    ~DeviceBuffer() { if (p) cudaFree(p); }
    void resize(size_t m)
    {
        if (m <= n && p) return;
        if (p) cudaFree(p);
        p = nullptr;
        cuda(cudaMalloc(&p, sizeof(T) * (m ? m : 1)), "cudaMalloc");
        n = m;
    }
    void upload(const T *host, size_t m)
    {
        resize(m);
        if (m) cuda(cudaMemcpy(p, host, sizeof(T) * m, cudaMemcpyHostToDevice), "cudaMemcpy");
    }
};
}  // namespace detail

namespace Scene {

// Scene/KDNode.h:26-98: SoA node arrays of a built tree.
class KDNode {
public:
    static const int MAX_LOWER_SIZE = 32;
    static const char LEAF = 0, X = 1, Y = 2, Z = 3;
    typedef int bitmap;
    typedef int amount;

    KDNode() = default;
    explicit KDNode(const kdgb_tree_view &v) : v_(v) {}

    char *GetInfoData() { return reinterpret_cast<char *>(v_.info); }
    float *GetSplitPositionData() { return v_.split; }
    float4 *GetAabbMinData() { return reinterpret_cast<float4 *>(v_.aabb_min); }
    float4 *GetAabbMaxData() { return reinterpret_cast<float4 *>(v_.aabb_max); }
    int *GetPrimitiveIndexData() { return v_.prim_index; }
    amount *GetPrimitiveAmountData() { return v_.bitmap; }
    bitmap *GetPrimitiveBitmapData() { return v_.bitmap; }
    int2 *GetChildrenData() { return reinterpret_cast<int2 *>(v_.children); }
    int GetSize() const { return v_.n_nodes; }

protected:
    kdgb_tree_view v_{};
};

// Scene/TriangleNode.h:18-34.
class TriangleNode : public KDNode {
public:
    TriangleNode() = default;
    explicit TriangleNode(const kdgb_tree_view &v) : KDNode(v) {}
    float *GetSurfaceAreaData() const { return v_.area; }
    int *GetParentData() const { return v_.parent; }
};

// Scene/CUDAMeshNode.h:20-41: device vertex/normal/colour/index buffers.
class CUDAMeshNode {
public:
    CUDAMeshNode() = default;
    // Vertices and normals as float3 (w = 1 / 0 like CopyVertices /
    // CopyNormals, CUDAMeshNode.cu:24-42), colours as uchar4.
    CUDAMeshNode(const std::vector<float3> &vertices, const std::vector<float3> &normals,
                 const std::vector<unsigned int> &indices)
    {
        std::vector<float4> v(vertices.size()), n(normals.size());
        for (size_t i = 0; i < v.size(); ++i) v[i] = make_float4(vertices[i].x, vertices[i].y, vertices[i].z, 1.0f);
        for (size_t i = 0; i < n.size(); ++i) n[i] = make_float4(normals[i].x, normals[i].y, normals[i].z, 0.0f);
        vertices_.upload(v.data(), v.size());
        normals_.upload(n.data(), n.size());
        std::vector<uchar4> c(vertices.size(), make_uchar4(180, 180, 180, 255));  // SetColor default
        colors_.upload(c.data(), c.size());
        indices_.upload(indices.data(), indices.size());
    }
    virtual ~CUDAMeshNode() = default;

    float4 *GetVertexData() const { return vertices_.p; }
    float4 *GetNormalData() const { return normals_.p; }
    uchar4 *GetColorData() const { return colors_.p; }
    unsigned int *GetIndexData() const { return indices_.p; }
    unsigned int GetSize() const { return (unsigned int)indices_.n; }
    unsigned int GetVertexCount() const { return (unsigned int)vertices_.n; }

protected:
    detail::DeviceBuffer<float4> vertices_, normals_;
    detail::DeviceBuffer<uchar4> colors_;
    detail::DeviceBuffer<unsigned int> indices_;
};

// Scene/OscCUDAMeshNode.h: an animated (detail+1)^2 height field in the x-z
// plane (OscCUDAMeshNode.cu:27-70 for the grid, :75-107 for the animation).
class OscCUDAMeshNode : public CUDAMeshNode {
public:
    OscCUDAMeshNode(float width, float depth, float height, int detail)
        : width_(width), depth_(depth), height_(height), detail_(detail) {}

    void Init()
    {
        if (vertices_.p) return;
        const unsigned d = detail_ + 1, size = d * d;
        const float ux = width_ / float(detail_), uz = depth_ / float(detail_);
        std::vector<float4> vert(size), norm(size, make_float4(0.0f, 1.0f, 0.0f, 0.0f));
        for (unsigned i = 0; i < d; ++i)
            for (unsigned j = 0; j < d; ++j)
                vert[i + j * d] = make_float4(i * ux - width_ * 0.5f, height_, j * uz - depth_ * 0.5f, 1.0f);
        std::vector<uchar4> col(size, make_uchar4(100, 200, 230, 128));
        std::vector<unsigned int> idx;
        idx.reserve(6u * detail_ * detail_);
        for (unsigned m = 0; m < (unsigned)detail_; ++m)
            for (unsigned n = 0; n < (unsigned)detail_; ++n) {
                idx.push_back(m + n * d); idx.push_back(m + (n + 1) * d); idx.push_back(m + 1 + n * d);
                idx.push_back(m + 1 + n * d); idx.push_back(m + (n + 1) * d); idx.push_back(m + 1 + (n + 1) * d);
            }
        vertices_.upload(vert.data(), vert.size());
        normals_.upload(norm.data(), norm.size());
        colors_.upload(col.data(), col.size());
        indices_.upload(idx.data(), idx.size());
    }

    // Handle(ProcessEventArg): advance by `approx_us` microseconds.
    void Handle(unsigned int approx_us, cudaStream_t s = 0)
    {
        time_ += approx_us;
        detail::check(kdgb_osc_update_surface(reinterpret_cast<float *>(vertices_.p),
                                              reinterpret_cast<float *>(normals_.p), detail_, height_,
                                              time_ / 700000.0f, s),
                      "OscCUDAMeshNode::Handle");
    }

private:
    float width_, depth_, height_;
    int detail_;
    unsigned int time_ = 0;
};

}  // namespace Scene

namespace Utils {
namespace CUDA {

// Utils/CUDA/GeometryList.h: concatenated triangle soup of all meshes.
class GeometryList {
public:
    // AddMesh(CUDAMeshNode*, model matrix) (GeometryList.cu:318-341); the
    // model matrix is row major and applied as Matrix44f * float4, the
    // normal matrix (row major 3x3, NULL = identity) to the normals.  Fills
    // the triangle buffer and the per-triangle normals n0/n1/n2 and colour
    // c0 (GeometryList.h:41-47).
    void AddMesh(const Scene::CUDAMeshNode &mesh, const float model[16] = nullptr,
                 const float normal_matrix[9] = nullptr, cudaStream_t s = 0)
    {
        const int32_t tris = (int32_t)mesh.GetSize() / 3;
        const size_t old = (size_t)size_;
        if ((size_t)(size_ + tris) > cap_) {
            const size_t cap = (size_t)(size_ + tris) * 2;
            grow(tri_, old * 9, cap * 9);
            grow(n0_, old * 4, cap * 4);
            grow(n1_, old * 4, cap * 4);
            grow(n2_, old * 4, cap * 4);
            grow(c0_, old * 4, cap * 4);
            cap_ = cap;
        }
        detail::check(kdgb_geometry_gather(reinterpret_cast<const float *>(mesh.GetVertexData()),
                                           (int32_t)mesh.GetVertexCount(), mesh.GetIndexData(), (int32_t)mesh.GetSize(),
                                           model, tri_.p + old * 9, s),
                      "GeometryList::AddMesh");
        detail::check(kdgb_geometry_gather_attributes(
                          reinterpret_cast<const float *>(mesh.GetNormalData()),
                          reinterpret_cast<const uint8_t *>(mesh.GetColorData()), (int32_t)mesh.GetVertexCount(),
                          mesh.GetIndexData(), (int32_t)mesh.GetSize(), normal_matrix, n0_.p + old * 4, n1_.p + old * 4,
                          n2_.p + old * 4, c0_.p + old * 4, s),
                      "GeometryList::AddMesh");
        size_ += tris;
    }
    void Clear() { size_ = 0; }
    int GetSize() const { return size_; }
    const float *GetTriangleData() const { return tri_.p; }
    const float *GetNormal0Data() const { return n0_.p; }
    const float *GetNormal1Data() const { return n1_.p; }
    const float *GetNormal2Data() const { return n2_.p; }
    const uint8_t *GetColor0Data() const { return c0_.p; }

private:
    template <class T>
    static void grow(detail::DeviceBuffer<T> &b, size_t keep, size_t n)
    {
        detail::DeviceBuffer<T> bigger;
        bigger.resize(n);
        if (keep) detail::cuda(cudaMemcpy(bigger.p, b.p, keep * sizeof(T), cudaMemcpyDeviceToDevice), "cudaMemcpy");
        std::swap(bigger.p, b.p);
        std::swap(bigger.n, b.n);
    }
    detail::DeviceBuffer<float> tri_, n0_, n1_, n2_;
    detail::DeviceBuffer<uint8_t> c0_;
    size_t cap_ = 0;
    int size_ = 0;
};

// Utils/CUDA/TriangleMap.h:31-83.
class TriangleMap {
public:
    enum LowerAlgorithm { BITMAP, BALANCED, SAH };
    enum SplitMethod { BOX, DIVIDE, SPLIT };

    explicit TriangleMap(GeometryList *geom) : geom_(geom)
    {
        kdgb_build_params_default(&p_);
        SetLowerAlgorithm(BITMAP);     // TriangleMap.cu:46-48
        SetPropagateBoundingBox(true);
        SetTraversalCost(24.0f);
    }
    ~TriangleMap() { if (tree_) kdgb_tree_destroy(tree_); }
    TriangleMap(const TriangleMap &) = delete;
    TriangleMap &operator=(const TriangleMap &) = delete;

    void Create(cudaStream_t s = 0)
    {
        p_.empty_space_threshold = EmptySpaceThreshold();
        if (tree_)
            detail::check(kdgb_rebuild(tree_, geom_->GetTriangleData(), geom_->GetSize(), &p_, s), "TriangleMap::Create");
        else
            detail::check(kdgb_build(geom_->GetTriangleData(), geom_->GetSize(), &p_, &tree_, s), "TriangleMap::Create");
        kdgb_build_stats st;
        kdgb_tree_stats(tree_, &st);
        constructionTime_ = st.build_ms;
    }

    LowerAlgorithm GetLowerAlgorithm() const { return lower_; }
    void SetLowerAlgorithm(const LowerAlgorithm l)
    {
        lower_ = l;
        p_.lower = l == SAH ? KDGB_LOWER_SAH : (l == BALANCED ? KDGB_LOWER_BALANCED : KDGB_LOWER_BITMAP);
    }
    float GetConstructionTime() const { return constructionTime_; }
    void SplitEmptySpace(const bool s) { p_.split_empty_space = s; }
    bool IsSplittingEmptySpace() const { return p_.split_empty_space != 0; }
    // SPLIT is stored and refused by Create(), where the reference throws
    // NotImplemented (TriangleMapUpperCreator.cu:551-552).
    void SetSplitMethod(const SplitMethod m)
    {
        p_.split_method = m == DIVIDE ? KDGB_SPLIT_DIVIDE : (m == SPLIT ? KDGB_SPLIT_SPLIT : KDGB_SPLIT_BOX);
    }
    SplitMethod GetSplitMethod() const
    {
        return p_.split_method == KDGB_SPLIT_DIVIDE ? DIVIDE : (p_.split_method == KDGB_SPLIT_SPLIT ? SPLIT : BOX);
    }
    void SetPropagateBoundingBox(const bool p) { p_.propagate_aabbs = p; }
    bool GetPropagateBoundingBox() const { return p_.propagate_aabbs != 0; }
    void SetTraversalCost(const float t) { p_.traversal_cost = t; }
    float GetTraversalCost() const { return p_.traversal_cost; }
    static void SetEmptySpaceThreshold(const float t) { EmptySpaceThreshold() = t; }

    GeometryList *GetGeometry() const { return geom_; }
    Scene::TriangleNode *GetNodes()
    {
        kdgb_tree_view v;
        detail::check(kdgb_tree_view_get(tree_, &v), "TriangleMap::GetNodes");
        nodes_ = Scene::TriangleNode(v);
        return &nodes_;
    }
    int *GetPrimitiveIndices()
    {
        kdgb_tree_view v;
        detail::check(kdgb_tree_view_get(tree_, &v), "TriangleMap::GetPrimitiveIndices");
        return v.prim_indices;
    }
    const kdgb_tree *Handle() const { return tree_; }
    kdgb_build_params &Params() { return p_; }

private:
    static float &EmptySpaceThreshold()
    {
        static float t = 0.35f;  // TriangleMapUpperCreator.cu:28
        return t;
    }
    GeometryList *geom_;
    kdgb_build_params p_;
    LowerAlgorithm lower_ = BITMAP;
    kdgb_tree *tree_ = nullptr;
    float constructionTime_ = 0.0f;
    Scene::TriangleNode nodes_;
};

// Utils/CUDA/IRayTracer.h:28-58.  Trace writes first-hit buffers (device
// pointers) instead of shading into an OpenGL canvas.
// What HostTrace found for one pixel: the shaded colour (the reference logs
// it as "Final color") and the pixel ray's first hit.
struct HostTraceResult {
    uchar4 color;
    int hit;      // triangle id, -1 = miss
    float t, u, v;
};

class IRayTracer {
public:
    enum IntersectionAlgorithm { MOELLER, WOOP };
    explicit IRayTracer(int tracer) { kdgb_trace_params_default(&p_); p_.tracer = tracer; }
    virtual ~IRayTracer() = default;

    virtual void Trace(const float *origins, const float *directions, int n, int *hit, float *t, float *u, float *v,
                       cudaStream_t s = 0) = 0;
    // Trace(IRenderCanvas*, uchar4* canvasData) (Raytracer.cu:295): the
    // shaded pixels of n rays (a width-wide image when Params().tile_width is
    // set) into canvasData, with Light() as the scene light.
    virtual void Trace(const float *origins, const float *directions, int n, uchar4 *canvasData,
                       cudaStream_t s = 0) = 0;

    // HostTrace(int x, int y, TriangleNode*) (IRayTracer.h:48;
    // Raytracer.cu:392-459, ShortStack.cu:323-351, BruteTracer.cu:174-199):
    // re-traces the ray of pixel (x, y) -- ray x + y * GetScreenWidth() of
    // the last Trace call's rays -- and returns its colour and first hit.
    // The reference runs its tracer function on the host; here the same
    // device tracer as Trace runs on that one ray and the result is copied
    // back (synchronises `s`).  `nodes` must be NULL or the traced map's
    // current GetNodes(): the map's own tree is what is traced.
    virtual HostTraceResult HostTrace(int x, int y, Scene::TriangleNode *nodes = nullptr, cudaStream_t s = 0) = 0;

    // The image width that maps (x, y) to a ray: Params().tile_width when it
    // is set, otherwise the width given here (the reference takes it from the
    // canvas, IRayTracer.cu:45-70).
    void SetScreenWidth(const int w) { screenWidth_ = w; }
    int GetScreenWidth() const { return p_.tile_width > 0 ? p_.tile_width : screenWidth_; }

    void SetIntersectionAlgorithm(const IntersectionAlgorithm a)
    {
        p_.intersection = a == WOOP ? KDGB_ISECT_WOOP : KDGB_ISECT_MOELLER;
    }
    IntersectionAlgorithm GetIntersectionAlgorithm() const
    {
        return p_.intersection == KDGB_ISECT_WOOP ? WOOP : MOELLER;
    }
    void SetLeafSkipping(const bool s) { p_.leaf_skipping = s; }
    bool GetLeafSkipping() const { return p_.leaf_skipping != 0; }
    float GetRenderTime() const { return renderTime_; }
    kdgb_trace_params &Params() { return p_; }
    kdgb_light &Light() { return light_; }

protected:
    void Remember(const float *o, const float *d, int n)
    {
        lastO_ = o;
        lastD_ = d;
        lastN_ = n;
    }
    // The device index of ray (x, y) of the last Trace; throws when there is
    // none.
    int PixelRay(int x, int y) const
    {
        const int w = GetScreenWidth();
        if (!lastO_ || w <= 0 || x < 0 || x >= w || y < 0)
            throw Core::Exception("IRayTracer::HostTrace: no traced image or pixel outside it");
        const int64_t id = (int64_t)x + (int64_t)y * w;
        if (id >= lastN_) throw Core::Exception("IRayTracer::HostTrace: pixel outside the last traced rays");
        return (int)id;
    }
    // Runs `first_hit` (one ray -> hit/t/u/v on the device) and `shade`
    // (one ray -> one RGBA pixel) for ray `id` and copies both back.
    template <class Hit, class Shade>
    HostTraceResult OnePixel(int id, Hit &&first_hit, Shade &&shade, cudaStream_t s)
    {
        detail::DeviceBuffer<float> buf;
        buf.resize(8);
        float *t = buf.p, *u = buf.p + 1, *v = buf.p + 2;
        int *hit = reinterpret_cast<int *>(buf.p + 3);
        uint8_t *rgba = reinterpret_cast<uint8_t *>(buf.p + 4);
        const float *o = lastO_ + 3 * (int64_t)id, *d = lastD_ + 3 * (int64_t)id;
        kdgb_trace_params p = p_;
        p.tile_width = 0;
        detail::check(first_hit(p, o, d, hit, t, u, v), "IRayTracer::HostTrace");
        detail::check(shade(p, o, d, rgba), "IRayTracer::HostTrace");
        float host[5];
        detail::cuda(cudaMemcpyAsync(host, buf.p, sizeof(host), cudaMemcpyDeviceToHost, s), "IRayTracer::HostTrace");
        detail::cuda(cudaStreamSynchronize(s), "IRayTracer::HostTrace");
        HostTraceResult r;
        r.t = host[0];
        r.u = host[1];
        r.v = host[2];
        std::memcpy(&r.hit, &host[3], 4);
        std::memcpy(&r.color, &host[4], 4);
        return r;
    }
    static void CheckNodes(const kdgb_tree *tree, Scene::TriangleNode *nodes)
    {
        if (!nodes) return;
        kdgb_tree_view v;
        detail::check(kdgb_tree_view_get(tree, &v), "IRayTracer::HostTrace");
        if (reinterpret_cast<int8_t *>(nodes->GetInfoData()) != v.info)
            throw Core::Exception("IRayTracer::HostTrace: nodes are not the traced map's current tree");
    }
    void TraceTree(const kdgb_tree *tree, bool propagate, const float *o, const float *d, int n, int *hit, float *t,
                   float *u, float *v, cudaStream_t s)
    {
        Remember(o, d, n);
        kdgb_trace_params p = p_;
        if (!propagate) p.leaf_skipping = 0;  // Raytracer.cu:313
        Timed([&] { return kdgb_trace(tree, &p, o, d, n, hit, t, u, v, s); }, "IRayTracer::Trace", s);
    }
    HostTraceResult HostTraceTree(const kdgb_tree *tree, bool propagate, const GeometryList *g, int x, int y,
                                  Scene::TriangleNode *nodes, cudaStream_t s)
    {
        CheckNodes(tree, nodes);
        const int id = PixelRay(x, y);
        return OnePixel(
            id,
            [&](kdgb_trace_params &p, const float *o, const float *d, int *hit, float *t, float *u, float *v) {
                if (!propagate) p.leaf_skipping = 0;
                return kdgb_trace(tree, &p, o, d, 1, hit, t, u, v, s);
            },
            [&](kdgb_trace_params &p, const float *o, const float *d, uint8_t *rgba) {
                return kdgb_trace_shaded(tree, &p, g->GetNormal0Data(), g->GetNormal1Data(), g->GetNormal2Data(),
                                         g->GetColor0Data(), &light_, 0, o, d, 1, rgba, s);
            },
            s);
    }
    template <class F>
    void Timed(F &&f, const char *where, cudaStream_t s)
    {
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        cudaEventRecord(e0, s);
        const int rc = f();
        cudaEventRecord(e1, s);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&renderTime_, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        detail::check(rc, where);
    }
    void ShadeTree(const kdgb_tree *tree, bool propagate, const GeometryList *g, const float *o, const float *d, int n,
                   uchar4 *canvas, cudaStream_t s)
    {
        Remember(o, d, n);
        kdgb_trace_params p = p_;
        if (!propagate) p.leaf_skipping = 0;
        Timed([&] {
            return kdgb_trace_shaded(tree, &p, g->GetNormal0Data(), g->GetNormal1Data(), g->GetNormal2Data(),
                                     g->GetColor0Data(), &light_, 0, o, d, n, reinterpret_cast<uint8_t *>(canvas), s);
        }, "IRayTracer::Trace", s);
    }
    kdgb_trace_params p_;
    kdgb_light light_ = DefaultLight();
    float renderTime_ = 0.0f;
    int screenWidth_ = 0;
    const float *lastO_ = nullptr, *lastD_ = nullptr;
    int lastN_ = 0;

private:
    static kdgb_light DefaultLight()
    {
        kdgb_light l;
        kdgb_light_default(&l);
        return l;
    }
};

class RayTracer : public IRayTracer {
public:
    explicit RayTracer(TriangleMap *map) : IRayTracer(KDGB_TRACER_RESTART), map_(map) {}
    void Trace(const float *o, const float *d, int n, int *hit, float *t, float *u, float *v, cudaStream_t s = 0) override
    {
        TraceTree(map_->Handle(), map_->GetPropagateBoundingBox(), o, d, n, hit, t, u, v, s);
    }
    void Trace(const float *o, const float *d, int n, uchar4 *canvas, cudaStream_t s = 0) override
    {
        ShadeTree(map_->Handle(), map_->GetPropagateBoundingBox(), map_->GetGeometry(), o, d, n, canvas, s);
    }
    HostTraceResult HostTrace(int x, int y, Scene::TriangleNode *nodes = nullptr, cudaStream_t s = 0) override
    {
        return HostTraceTree(map_->Handle(), map_->GetPropagateBoundingBox(), map_->GetGeometry(), x, y, nodes, s);
    }

private:
    TriangleMap *map_;
};

class ShortStack : public IRayTracer {
public:
    explicit ShortStack(TriangleMap *map) : IRayTracer(KDGB_TRACER_SHORTSTACK), map_(map) {}
    void Trace(const float *o, const float *d, int n, int *hit, float *t, float *u, float *v, cudaStream_t s = 0) override
    {
        TraceTree(map_->Handle(), map_->GetPropagateBoundingBox(), o, d, n, hit, t, u, v, s);
    }
    void Trace(const float *o, const float *d, int n, uchar4 *canvas, cudaStream_t s = 0) override
    {
        ShadeTree(map_->Handle(), map_->GetPropagateBoundingBox(), map_->GetGeometry(), o, d, n, canvas, s);
    }
    HostTraceResult HostTrace(int x, int y, Scene::TriangleNode *nodes = nullptr, cudaStream_t s = 0) override
    {
        return HostTraceTree(map_->Handle(), map_->GetPropagateBoundingBox(), map_->GetGeometry(), x, y, nodes, s);
    }

private:
    TriangleMap *map_;
};

// BruteTracer (BruteTracer.cu): every triangle of the GeometryList, no tree.
class BruteTracer : public IRayTracer {
public:
    explicit BruteTracer(GeometryList *geom) : IRayTracer(KDGB_TRACER_BRUTE), geom_(geom) {}
    void Trace(const float *o, const float *d, int n, int *hit, float *t, float *u, float *v, cudaStream_t s = 0) override
    {
        Remember(o, d, n);
        detail::check(kdgb_trace_brute_ex(geom_->GetTriangleData(), geom_->GetSize(), &p_, o, d, n, hit, t, u, v, s),
                      "BruteTracer::Trace");
    }
    void Trace(const float *o, const float *d, int n, uchar4 *canvas, cudaStream_t s = 0) override
    {
        Remember(o, d, n);
        const GeometryList *g = geom_;
        Timed([&] {
            return kdgb_trace_brute_shaded(g->GetTriangleData(), g->GetSize(), &p_, g->GetNormal0Data(),
                                           g->GetNormal1Data(), g->GetNormal2Data(), g->GetColor0Data(), &light_, 0, o,
                                           d, n, reinterpret_cast<uint8_t *>(canvas), s);
        }, "BruteTracer::Trace", s);
    }
    // BruteTracer::HostTrace (BruteTracer.cu:174-199) tests every triangle;
    // `nodes` is not used, as in the reference.
    HostTraceResult HostTrace(int x, int y, Scene::TriangleNode * = nullptr, cudaStream_t s = 0) override
    {
        const GeometryList *g = geom_;
        return OnePixel(
            PixelRay(x, y),
            [&](kdgb_trace_params &p, const float *o, const float *d, int *hit, float *t, float *u, float *v) {
                return kdgb_trace_brute_ex(g->GetTriangleData(), g->GetSize(), &p, o, d, 1, hit, t, u, v, s);
            },
            [&](kdgb_trace_params &p, const float *o, const float *d, uint8_t *rgba) {
                return kdgb_trace_brute_shaded(g->GetTriangleData(), g->GetSize(), &p, g->GetNormal0Data(),
                                               g->GetNormal1Data(), g->GetNormal2Data(), g->GetColor0Data(), &light_,
                                               0, o, d, 1, rgba, s);
            },
            s);
    }

private:
    GeometryList *geom_;
};

}  // namespace CUDA
}  // namespace Utils
}  // namespace OpenEngine
