// Drives the C++ plugin mirror (include/gridrt_rtp.hpp) the way the
// reference's Context does: build a Geometry through the builder, then trace
// rays one by one through the virtual per-ray calls and in one batch.
// Reads rays and geometry from binary files, writes hits for the Python test.
// With a camera file (an rtg_camera followed by the light position, 3
// float32) it also renders that frame with GpuFrameRenderer and then as a
// stream of frames through GpuFrameStream, and reports the words that differ.
//   rtp_adapter_check <verts.f32> <tris.i32> <rays.f32> <out_prefix> [camera.bin]
#include <cstdio>
#include <cstring>
#include <fstream>
#include <vector>

#include "gridrt_rtp.hpp"

using namespace gridrt;

template <class T>
static std::vector<T> load(const char* path) {
    std::ifstream f(path, std::ios::binary | std::ios::ate);
    std::vector<T> v((size_t)f.tellg() / sizeof(T));
    f.seekg(0);
    f.read(reinterpret_cast<char*>(v.data()), (std::streamsize)(v.size() * sizeof(T)));
    return v;
}

int main(int argc, char** argv) {
    if (argc != 5 && argc != 6) return 2;
    std::vector<float> verts = load<float>(argv[1]);
    std::vector<int32_t> tris = load<int32_t>(argv[2]);
    std::vector<float> rays = load<float>(argv[3]);
    rt::Geometry g;
    for (size_t i = 0; i + 2 < verts.size(); i += 3) g.vertices.emplace_back(verts[i], verts[i + 1], verts[i + 2]);
    for (size_t t = 0; t + 2 < tris.size(); t += 3) g.triDesc.push_back({{(uint32_t)tris[t], (uint32_t)tris[t + 1], (uint32_t)tris[t + 2]}});
    rtp::UniformGridAccStructBuilder builder(4);
    builder.buildGeometry(&g);
    if (builder.lastStatus() != RTG_OK) {
        std::fprintf(stderr, "build failed: %s\n", rtg_last_error());
        return 1;
    }
    auto* acc = static_cast<rtp::UniformGridAccStruct*>(g.accStruct.get());
    rt::Instance inst;
    inst.geometry = &g;
    const size_t n = rays.size() / 8;
    std::vector<rt::Ray> rv(n);
    for (size_t i = 0; i < n; ++i) {
        const float* q = &rays[8 * i];
        rv[i].orig = rt::vec3f(q[0], q[1], q[2]);
        rv[i].tnear = q[3];
        rv[i].dir = rt::vec3f(q[4], q[5], q[6]);
        rv[i].tfar = q[7];
    }
    // per-ray virtual calls (as IAccStruct::traceNearestInstance makes them)
    std::vector<float> single(4 * n), batch(4 * n);
    std::vector<uint8_t> any_single(n);
    rt::IAccStruct* base = acc;
    for (size_t i = 0; i < n; ++i) {
        rt::Ray r = rv[i];
        rt::Hit h;
        base->traceNearestGeometry(inst, r, h);
        int32_t id = h.instance ? (int32_t)h.triangleId : -1;
        std::memcpy(&single[4 * i], &id, 4);
        single[4 * i + 1] = h.instance ? h.distance : 0.f;
        single[4 * i + 2] = h.instance ? h.v1Coord : 0.f;
        single[4 * i + 3] = h.instance ? h.v2Coord : 0.f;
        rt::Ray r2 = rv[i];
        any_single[i] = base->traceAnyGeometry(inst, r2, h) ? 1 : 0;
    }
    std::vector<rt::Hit> hits;
    acc->traceNearestBatch(inst, rv, hits);
    for (size_t i = 0; i < n; ++i) {
        int32_t id = hits[i].instance ? (int32_t)hits[i].triangleId : -1;
        std::memcpy(&batch[4 * i], &id, 4);
        batch[4 * i + 1] = hits[i].instance ? hits[i].distance : 0.f;
        batch[4 * i + 2] = hits[i].instance ? hits[i].v1Coord : 0.f;
        batch[4 * i + 3] = hits[i].instance ? hits[i].v2Coord : 0.f;
    }
    std::vector<uint8_t> any_batch;
    acc->traceAnyBatch(rv, any_batch);
    // the scene level: one identity instance of the geometry
    rtp::InstancedScene scene;
    scene.buildInstance(std::vector<rt::Instance>{inst});
    std::vector<rt::Hit> ihits;
    scene.traceNearestInstance(rv, ihits);
    if (scene.lastStatus() != RTG_OK) {
        std::fprintf(stderr, "instance trace failed: %s\n", rtg_last_error());
        return 1;
    }
    std::vector<float> inst_hits(4 * n);
    for (size_t i = 0; i < n; ++i) {
        int32_t id = ihits[i].instance ? (int32_t)ihits[i].triangleId : -1;
        std::memcpy(&inst_hits[4 * i], &id, 4);
        inst_hits[4 * i + 1] = ihits[i].instance ? ihits[i].distance : 0.f;
        inst_hits[4 * i + 2] = ihits[i].instance ? ihits[i].v1Coord : 0.f;
        inst_hits[4 * i + 3] = ihits[i].instance ? ihits[i].v2Coord : 0.f;
    }
    auto save = [&](const char* suffix, const void* data, size_t bytes) {
        std::string path = std::string(argv[4]) + suffix;
        std::ofstream(path, std::ios::binary).write(static_cast<const char*>(data), (std::streamsize)bytes);
    };
    save(".single.f32", single.data(), single.size() * 4);
    save(".batch.f32", batch.data(), batch.size() * 4);
    save(".any_single.u8", any_single.data(), any_single.size());
    save(".any_batch.u8", any_batch.data(), any_batch.size());
    save(".inst.f32", inst_hits.data(), inst_hits.size() * 4);
    long long frame_diff = -1;
    if (argc == 6) {
        std::vector<uint8_t> camfile = load<uint8_t>(argv[5]);
        if (camfile.size() != sizeof(rtg_camera) + 12) return 2;
        rtg_camera cam;
        float light[3];
        std::memcpy(&cam, camfile.data(), sizeof(cam));
        std::memcpy(light, camfile.data() + sizeof(cam), 12);
        std::vector<rtg_hit> ref_hits;
        std::vector<uint8_t> ref_occ;
        if (rtp::GpuFrameRenderer::render(*acc, cam, light, ref_hits, ref_occ) != RTG_OK) {
            std::fprintf(stderr, "frame failed: %s\n", rtg_last_error());
            return 1;
        }
        rtp::GpuFrameStream frames(*acc);
        frame_diff = 0;
        uint64_t prev = 0, t = 0;
        const std::vector<rtg_hit>* h = nullptr;
        const std::vector<uint8_t>* o = nullptr;
        auto compare = [&]() {
            for (size_t i = 0; i < ref_hits.size(); ++i) {
                frame_diff += std::memcmp(&(*h)[i], &ref_hits[i], sizeof(rtg_hit)) != 0;
                frame_diff += (*o)[i] != ref_occ[i];
            }
        };
        for (int f = 0; f < 4; ++f) {
            if (frames.begin(cam, light, &t) != RTG_OK) return 1;
            if (f > 0) {
                if (frames.finish(prev, &h, &o) != RTG_OK) return 1;
                compare();
            }
            prev = t;
        }
        if (frames.finish(prev, &h, &o) != RTG_OK) return 1;
        compare();
    }
    rtg_grid_info gi = acc->gridInfo();
    std::printf("{\"res\": [%d, %d, %d], \"nrefs\": %lld, \"frame_diff\": %lld}\n", gi.res[0], gi.res[1], gi.res[2],
                (long long)gi.nrefs, frame_diff);
    return 0;
}
