// krr_wavefront_pass.hpp — header-only C++ front end of the C ABI for host
// applications written in C++, shaped like the reference's render pass
// (class WavefrontPathTracer : public RenderPass,
// src/render/wavefront/integrator.h:24-104): constructed from the pass's
// JSON parameters, then setScene / resize / beginFrame / render, plus the
// stage methods and queue views that PPG-style subclasses call
// (src/misc/render/ppg/integrator.h:13).  Errors throw krr::Error carrying
// the library's status and message (the reference logs and terminates,
// src/util/check.h:8-51).
//
// A host binds it into its own RenderPass hierarchy by holding one
// krr::WavefrontPass and forwarding its virtuals (resize, setScene,
// beginFrame, render).  Only the C ABI crosses the library boundary.
#pragma once

#include <stdexcept>
#include <string>

#include "krr_gb300.h"

namespace krr {

class Error : public std::runtime_error {
public:
    Error(int status, const std::string &what) : std::runtime_error(what), status_(status) {}
    int status() const { return status_; }

private:
    int status_;
};

inline void check(int status, const char *call) {
    if (status != KRR_OK)
        throw Error(status, std::string(call) + ": " + krr_status_string(status) + ": " + krr_last_error());
}

class WavefrontPass {
public:
    // from_json (integrator.h:85-103): "nee", "enable_medium", "max_depth",
    // "rr", "enable_clamp", "clamp_max"; "{}" gives the defaults.
    explicit WavefrontPass(const std::string &params_json = "{}") {
        check(krr_wf_create_json(params_json.c_str(), &pass_), "krr_wf_create_json");
    }
    ~WavefrontPass() { krr_wf_destroy(pass_); }
    WavefrontPass(const WavefrontPass &) = delete;
    WavefrontPass &operator=(const WavefrontPass &) = delete;

    static const char *getName() { return "WavefrontPathTracer"; }

    void setParams(const std::string &params_json) {
        check(krr_wf_set_params_json(pass_, params_json.c_str()), "krr_wf_set_params_json");
    }
    krr_wf_params params() const {
        krr_wf_params p;
        check(krr_wf_get_params(pass_, &p), "krr_wf_get_params");
        return p;
    }
    // RenderPass virtuals (integrator.cpp:181-267)
    void setScene(const krr_scene_desc &scene, void *stream) {
        check(krr_wf_set_scene(pass_, &scene, stream), "krr_wf_set_scene");
    }
    void resize(int width, int height) { check(krr_wf_resize(pass_, width, height), "krr_wf_resize"); }
    void beginFrame(int64_t frame_index, const krr_camera_desc &camera, void *stream) {
        check(krr_wf_begin_frame(pass_, frame_index, &camera, stream), "krr_wf_begin_frame");
    }
    // float4 RGBA per pixel, row 0 at the top
    void render(float *d_rgba, void *stream) { check(krr_wf_render(pass_, d_rgba, stream), "krr_wf_render"); }

    // stage methods (integrator.cpp:50-164)
    void generateCameraRays(void *stream) {
        check(krr_wf_generate_camera_rays(pass_, stream), "krr_wf_generate_camera_rays");
    }
    void traceClosest(int depth, void *stream) {
        check(krr_wf_trace_closest(pass_, depth, stream), "krr_wf_trace_closest");
    }
    void handleHit(void *stream) { check(krr_wf_handle_hit(pass_, stream), "krr_wf_handle_hit"); }
    void handleMiss(void *stream) { check(krr_wf_handle_miss(pass_, stream), "krr_wf_handle_miss"); }
    void generateScatterRays(int depth, void *stream) {
        check(krr_wf_generate_scatter_rays(pass_, depth, stream), "krr_wf_generate_scatter_rays");
    }
    void traceShadow(void *stream) { check(krr_wf_trace_shadow(pass_, stream), "krr_wf_trace_shadow"); }
    // SoA planes of a queue (workqueue.h:159-359): plane c of item i at base + 4 * (c * capacity + i)
    const float *queue(int kind, int *channels, int *capacity) const {
        const float *base = nullptr;
        check(krr_wf_queue_view(pass_, kind, &base, channels, capacity), "krr_wf_queue_view");
        return base;
    }
    // device error flags since the last call (see krr_wf_device_errors)
    uint32_t deviceErrors(void *stream) {
        uint32_t f = 0;
        check(krr_wf_device_errors(pass_, &f, stream), "krr_wf_device_errors");
        return f;
    }
    krr_wf *handle() const { return pass_; }

private:
    krr_wf *pass_ = nullptr;
};

}  // namespace krr
