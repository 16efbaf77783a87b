// The RenderPass binding a maintainer adds to the host application: a
// RenderPass subclass registered by name that holds a krr::WavefrontPass and
// forwards its virtuals; compiled here against host_stub.h.
#pragma once

#include "host_stub.h"
#include "krr_wavefront_pass.hpp"

class WavefrontPathTracerGB300 : public RenderPass {
public:
    explicit WavefrontPathTracerGB300(const json &params) : pass(params) {}
    std::string getName() const override { return krr::WavefrontPass::getName(); }
    void setScene(Scene::SharedPtr scene) override {
        RenderPass::setScene(scene);
        pass.setScene(scene->desc, stream);
    }
    void resize(const Vector2i &size) override {
        RenderPass::resize(size);
        pass.resize(size[0], size[1]);
    }
    void beginFrame(RenderContext *ctx) override {
        RenderPass::beginFrame(ctx);
        stream = ctx->stream;
        pass.beginFrame(getFrameIndex(), mScene->camera, stream);
    }
    void render(RenderContext *ctx) override { pass.render(ctx->color, ctx->stream); }
    // stage methods for PPG-style subclasses
    void traceClosest(int depth) { pass.traceClosest(depth, stream); }
    void handleHit() { pass.handleHit(stream); }
    void handleMiss() { pass.handleMiss(stream); }
    void generateScatterRays(int depth) { pass.generateScatterRays(depth, stream); }
    void traceShadow() { pass.traceShadow(stream); }
    krr::WavefrontPass pass;

private:
    void *stream = nullptr;
};
