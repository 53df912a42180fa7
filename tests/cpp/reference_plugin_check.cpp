// Drives the reference-side binding (include/gridrt_reference_plugin.hpp)
// compiled against the reference's own headers, beside the reference's own
// CPU plugin pair (rtp::UniformGridAccStructBuilder / UniformGridAccStruct,
// compiled from the reference's sources into oracle/_ref).  Two rt::Geometry
// objects with the same vertices and triangles are built, one by each
// builder through the rt::IAccStructBuilder interface; every ray is then
// prepared the way IAccStruct::traceNearestInstance prepares it
// (src/rtcore/IAccStruct.cpp:29-50: tnear = ray epsilon, tfar = MAX_VALUE,
// Ray::update, clip against the structure's bounding box) and traced through
// the rt::IAccStruct interface of both.  Prints one JSON line.
//
// Without a GPU the GPU builder must fail the reference's way (silently: the
// geometry still gets a structure, which reports no hit and leaves the hit
// record as it was); with one, the two plugins' hits are compared.
//   reference_plugin_check <verts.f32> <tris.i32> <rays.f32> <k> <out_prefix>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include <rt/AabbIntersection.h>
#include <rtp/UniformGridAccStruct.h>
#include <rtp/UniformGridAccStructBuilder.h>

#include "gridrt_reference_plugin.hpp"

template <class T>
static std::vector<T> load(const char* path) {
    std::ifstream f(path, std::ios::binary | std::ios::ate);
    std::vector<T> v((size_t)f.tellg() / sizeof(T));
    f.seekg(0);
    f.read(reinterpret_cast<char*>(v.data()), (std::streamsize)(v.size() * sizeof(T)));
    return v;
}

static void fill(rt::Geometry& g, const std::vector<float>& verts, const std::vector<int32_t>& tris) {
    for (size_t i = 0; i + 2 < verts.size(); i += 3) g.vertices.push_back(vr::vec3f(verts[i], verts[i + 1], verts[i + 2]));
    for (size_t t = 0; t + 2 < tris.size(); t += 3) {
        rt::TriDesc d;
        for (int j = 0; j < 3; ++j) d.v[j] = (uint32)tris[t + j];
        d.material = NULL;
        g.triDesc.push_back(d);
        // the CPU plugin tests TriAccel records (PrimitiveBuilder::storeValidTriangle)
        rt::TriAccel a;
        a.buildFrom(g.vertices[d.v[0]], g.vertices[d.v[1]], g.vertices[d.v[2]]);
        a.triangleId = (uint32)(g.triDesc.size() - 1);
        g.triAccel.push_back(a);
    }
}

// IAccStruct::traceNearestInstance's per-ray preparation, then the
// structure's traceNearestGeometry.  False when the ray misses the box.
static bool trace(rt::IAccStruct* acc, const rt::Instance& inst, const float* q, rt::Hit& hit) {
    rt::Ray ray;
    ray.orig.set(q[0], q[1], q[2]);
    ray.dir.set(q[4], q[5], q[6]);
    ray.tnear = 2e-4f;                      // Context::getRayEpsilon default (src/rtcore/Context.cpp:505)
    ray.tfar = vr::Mathf::MAX_VALUE;
    ray.update();
    hit.instance = NULL;
    hit.distance = vr::Mathf::MAX_VALUE;
    if (!rt::AabbIntersection::clipRay(acc->getBoundingBox(), ray)) return false;
    acc->traceNearestGeometry(inst, ray, hit);
    return true;
}

int main(int argc, char** argv) {
    if (argc != 6) return 2;
    std::vector<float> verts = load<float>(argv[1]);
    std::vector<int32_t> tris = load<int32_t>(argv[2]);
    std::vector<float> rays = load<float>(argv[3]);
    const int k = std::atoi(argv[4]);
    const size_t n = rays.size() / 8;

    vr::ref_ptr<rt::Geometry> cpu_geom = new rt::Geometry;
    vr::ref_ptr<rt::Geometry> gpu_geom = new rt::Geometry;
    fill(*cpu_geom, verts, tris);
    fill(*gpu_geom, verts, tris);

    // the reference's own builder hard-codes 6 cells per triangle
    vr::ref_ptr<rt::IAccStructBuilder> cpu_builder = new rtp::UniformGridAccStructBuilder;
    rtp::GpuUniformGridAccStructBuilder* gb = new rtp::GpuUniformGridAccStructBuilder(k, 0);
    vr::ref_ptr<rt::IAccStructBuilder> gpu_builder = gb;
    cpu_builder->buildGeometry(cpu_geom.get());
    gpu_builder->buildGeometry(gpu_geom.get());
    const int gpu_status = (int)gb->lastStatus();
    const bool gpu_has_struct = gpu_geom->accStruct.get() != NULL;
    rtp::GpuUniformGridAccStruct* gacc = dynamic_cast<rtp::GpuUniformGridAccStruct*>(gpu_geom->accStruct.get());
    const bool gpu_ok = gpu_status == RTG_OK && gacc && gacc->built();

    rt::Instance cpu_inst, gpu_inst;
    cpu_inst.geometry = cpu_geom.get();
    gpu_inst.geometry = gpu_geom.get();
    std::vector<float> cpu_out(4 * n, 0.f), gpu_out(4 * n, 0.f);
    long cpu_hits = 0, gpu_hits = 0, untouched = 0, same_id = 0, same_bits = 0, instance_ok = 0;
    for (size_t i = 0; i < n; ++i) {
        const float* q = &rays[8 * i];
        rt::Hit hc, hg;
        std::memset(&hc, 0, sizeof(hc));
        std::memset(&hg, 0, sizeof(hg));
        trace(cpu_geom->accStruct.get(), cpu_inst, q, hc);
        const bool cpu_hit = hc.instance != NULL;
        int32_t cid = cpu_hit ? (int32_t)hc.triangleId : -1;
        cpu_out[4 * i] = *reinterpret_cast<float*>(&cid);
        cpu_out[4 * i + 1] = hc.distance;
        cpu_out[4 * i + 2] = hc.v1Coord;
        cpu_out[4 * i + 3] = hc.v2Coord;
        cpu_hits += cpu_hit;

        hg.triangleId = 0xdeadbeefu;          // must survive a trace that finds nothing
        trace(gpu_geom->accStruct.get(), gpu_inst, q, hg);
        const bool gpu_hit = hg.instance != NULL;
        if (!gpu_hit && hg.triangleId == 0xdeadbeefu) ++untouched;
        int32_t gid = gpu_hit ? (int32_t)hg.triangleId : -1;
        gpu_out[4 * i] = *reinterpret_cast<float*>(&gid);
        gpu_out[4 * i + 1] = hg.distance;
        gpu_out[4 * i + 2] = hg.v1Coord;
        gpu_out[4 * i + 3] = hg.v2Coord;
        gpu_hits += gpu_hit;
        if (gpu_hit && hg.instance == &gpu_inst) ++instance_ok;
        if (gid == cid) {
            ++same_id;
            if (gpu_hit && std::memcmp(&gpu_out[4 * i + 1], &cpu_out[4 * i + 1], 12) == 0) ++same_bits;
        }
    }
    std::string p = argv[5];
    std::ofstream(p + ".cpu.f32", std::ios::binary).write(reinterpret_cast<const char*>(cpu_out.data()),
                                                          (std::streamsize)(cpu_out.size() * sizeof(float)));
    std::ofstream(p + ".gpu.f32", std::ios::binary).write(reinterpret_cast<const char*>(gpu_out.data()),
                                                          (std::streamsize)(gpu_out.size() * sizeof(float)));
    std::printf("{\"rays\": %zu, \"gpu_ok\": %s, \"gpu_status\": %d, \"gpu_has_struct\": %s, \"cpu_hits\": %ld, "
                "\"gpu_hits\": %ld, \"gpu_untouched\": %ld, \"same_id\": %ld, \"same_bits\": %ld, "
                "\"instance_ok\": %ld}\n",
                n, gpu_ok ? "true" : "false", gpu_status, gpu_has_struct ? "true" : "false", cpu_hits, gpu_hits,
                untouched, same_id, same_bits, instance_ok);
    return 0;
}
