// Minimal stand-ins for the host application's types that a RenderPass
// binding touches (the reference's RenderPass, src/core/renderpass.h:138-200;
// RenderPassFactory, :240-273; a scene reduced to the description the C ABI
// takes).  Test code only: the real binding compiles against the host's own
// headers.
#pragma once

#include <functional>
#include <map>
#include <memory>
#include <string>

#include "krr_gb300.h"

struct Vector2i {
    int x = 0, y = 0;
    int operator[](int i) const { return i == 0 ? x : y; }
};

// The host's per-frame context: the colour target and the CUDA stream.
struct RenderContext {
    float *color = nullptr;   // float4 RGBA device buffer
    void *stream = nullptr;
};

// The host's scene, already converted to the C ABI's description.
struct Scene {
    using SharedPtr = std::shared_ptr<Scene>;
    krr_scene_desc desc{};
    krr_camera_desc camera{};
};

using json = std::string;   // the pass's `params` object as JSON text

class RenderPass {
public:
    using SharedPtr = std::shared_ptr<RenderPass>;
    virtual ~RenderPass() = default;
    virtual void resize(const Vector2i &size) { mFrameSize = size; }
    virtual void setScene(Scene::SharedPtr scene) { mScene = scene; }
    virtual void beginFrame(RenderContext *) { ++mFrameIndex; }
    virtual void render(RenderContext *) {}
    virtual void endFrame(RenderContext *) {}
    virtual std::string getName() const { return "RenderPass"; }
    int getFrameIndex() const { return mFrameIndex; }   // 1-based once a frame began
    Vector2i getFrameSize() const { return mFrameSize; }

protected:
    Vector2i mFrameSize;
    int mFrameIndex = 0;
    Scene::SharedPtr mScene;
};

// Passes are made by name from the `passes[]` entries of a configuration
// (RenderPassFactory::deserizeInstance, src/main/renderer.cpp:274-286).
struct RenderPassFactory {
    using Maker = std::function<RenderPass::SharedPtr(const json &)>;
    static std::map<std::string, Maker> &registry() {
        static std::map<std::string, Maker> r;
        return r;
    }
    static RenderPass::SharedPtr deserizeInstance(const std::string &name, const json &params) {
        auto it = registry().find(name);
        return it == registry().end() ? nullptr : it->second(params);
    }
};

#define KRR_REGISTER_PASS_DEF(T)                                                        \
    static const bool T##_registered = [] {                                             \
        RenderPassFactory::registry()[#T] = [](const json &p) {                         \
            return std::static_pointer_cast<RenderPass>(std::make_shared<T>(p));        \
        };                                                                              \
        return true;                                                                    \
    }()
