// Drives WavefrontPathTracerGB300 through the host's RenderPass interface,
// for the integration tests: the pass is made by name from its JSON
// parameters, then setScene / resize / beginFrame / render.
#include <cstring>

#include "wavefront_gb300_pass.h"

KRR_REGISTER_PASS_DEF(WavefrontPathTracerGB300);

extern "C" int shim_params(const char *params_json, krr_wf_params *out, char *name, int name_cap) {
    try {
        RenderPass::SharedPtr p = RenderPassFactory::deserizeInstance("WavefrontPathTracerGB300", params_json);
        if (!p) return -1;
        std::strncpy(name, p->getName().c_str(), name_cap - 1);
        name[name_cap - 1] = 0;
        *out = static_cast<WavefrontPathTracerGB300 &>(*p).pass.params();
        return 0;
    } catch (const krr::Error &e) {
        return e.status();
    }
}

// Renders frames 1..frames (the host's frame counter) and leaves the last in d_out.
extern "C" int shim_render(const char *params_json, const krr_scene_desc *scene,
                           const krr_camera_desc *camera, int width, int height, int frames,
                           float *d_out) {
    try {
        RenderPass::SharedPtr p = RenderPassFactory::deserizeInstance("WavefrontPathTracerGB300", params_json);
        if (!p) return -1;
        auto sc = std::make_shared<Scene>();
        sc->desc = *scene;
        sc->camera = *camera;
        p->setScene(sc);
        p->resize(Vector2i{width, height});
        RenderContext ctx{d_out, nullptr};
        for (int f = 0; f < frames; ++f) {
            p->beginFrame(&ctx);
            p->render(&ctx);
            p->endFrame(&ctx);
        }
        return static_cast<WavefrontPathTracerGB300 &>(*p).pass.deviceErrors(nullptr) ? -2 : 0;
    } catch (const krr::Error &e) {
        return e.status();
    }
}
