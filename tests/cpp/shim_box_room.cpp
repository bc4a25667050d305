// Renders a small box room through mitrace::Tracer (the C++ shim with the
// reference Tracer's shape) while a second thread polls GetStats/IsDone, as
// MiTrace's StatThread does (src/main.cpp:41-77).  Prints one line:
//   ok <mean r> <mean g> <mean b> <rays> <samples> <progress>
#include <chrono>
#include <cstdio>
#include <memory>
#include <thread>
#include <vector>

#include "mitrace/Tracer.hpp"

static void quad(std::vector<float>& p, std::vector<float>& n, const float a[3], const float b[3],
                 const float c[3], const float d[3], const float nn[3])
{
    const float* tri[6] = {a, b, c, a, c, d};
    for (const float* v : tri) {
        p.insert(p.end(), v, v + 3);
        n.insert(n.end(), nn, nn + 3);
    }
}

int main(int argc, char** argv)
{
    std::vector<float> pos, nrm;
    const float f0[3] = {-1, 0, -1}, f1[3] = {-1, 0, 1}, f2[3] = {1, 0, 1}, f3[3] = {1, 0, -1}, up[3] = {0, 1, 0};
    const float b0[3] = {-1, 0, -1}, b1[3] = {1, 0, -1}, b2[3] = {1, 2, -1}, b3[3] = {-1, 2, -1}, fw[3] = {0, 0, 1};
    quad(pos, nrm, f0, f1, f2, f3, up);
    quad(pos, nrm, b0, b1, b2, b3, fw);
    mt_mesh_desc mesh{};
    mesh.num_triangles = static_cast<uint32_t>(pos.size() / 9);
    mesh.positions = pos.data();
    mesh.normals = nrm.data();
    mt_material_desc mat{};
    const float base[4] = {0.73f, 0.73f, 0.73f, 1.0f};
    for (int i = 0; i < 4; ++i) mat.base_color_factor[i] = base[i];
    mat.normal_scale = 1.0f;
    mat.roughness_factor = 1.0f;
    mat.base_color_tex = mat.metallic_roughness_tex = mat.normal_tex = mat.occlusion_tex = mat.emissive_tex = -1;
    mt_instance_desc inst{};
    for (int i = 0; i < 16; ++i) inst.transform[i] = (i % 5 == 0) ? 1.0f : 0.0f;
    mt_light_desc light{};
    light.type = MT_LIGHT_POINT;
    light.position[1] = 1.9f;
    light.color[0] = light.color[1] = light.color[2] = 20.0f;
    light.point_size = 0.05f;
    mt_scene_desc scene{};
    scene.num_meshes = 1;
    scene.meshes = &mesh;
    scene.num_instances = 1;
    scene.instances = &inst;
    scene.num_materials = 1;
    scene.materials = &mat;
    scene.num_lights = 1;
    scene.lights = &light;
    for (int i = 0; i < 16; ++i) scene.camera.camera_to_world[i] = (i % 5 == 0) ? 1.0f : 0.0f;
    scene.camera.camera_to_world[13] = 1.0f;
    scene.camera.camera_to_world[14] = 3.4f;
    scene.camera.yfov = 0.6981317f;
    scene.camera.aspect = 1.0f;
    scene.env_texture = -1;
    mt_config cfg;
    mt_config_defaults(&cfg);
    cfg.samples = 16;
    cfg.ev_exposure = 0.0f;

    auto buffer = std::make_shared<mitrace::RenderBuffer>(64, 64);
    try {
        mitrace::Tracer tracer(buffer, scene, cfg);
        tracer.StartRender();
        std::thread stat([&] {
            while (!tracer.IsDone()) {
                (void)tracer.GetStats();
                std::this_thread::sleep_for(std::chrono::milliseconds(1));
            }
        });
        tracer.WaitForRender();
        stat.join();
        const auto st = tracer.GetStats();
        double m[3] = {0, 0, 0};
        for (unsigned y = 0; y < 64; ++y)
            for (unsigned x = 0; x < 64; ++x) {
                float c[3];
                buffer->GetPixel(x, y, c);
                for (int k = 0; k < 3; ++k) m[k] += c[k] / (64.0 * 64.0);
            }
        if (argc > 1) {  // RenderBuffer::SaveToFilePNG / SaveToFileHDR
            buffer->SaveToFilePNG(std::string(argv[1]) + ".png");
            buffer->SaveToFileHDR(std::string(argv[1]) + ".hdr");
        }
        std::printf("ok %.6f %.6f %.6f %zu %zu %.3f\n", m[0], m[1], m[2], st.rays, st.samples, st.progress);
    } catch (const std::exception& e) {
        std::printf("error %s\n", e.what());
        return 1;
    }
    return 0;
}
