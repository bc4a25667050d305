// Tracer.hpp - C++ drop-in with the shape of MiTrace's Tracer::Tracer
// (src/Tracer/Tracer.hpp:19-129) over the C ABI in mitrace_gpu.h.
//
// Header-only.  The reference's Tracer reads the global Config and a
// Scene::Scene; this one takes the same data explicitly: an mt_config (the
// hot-path fields of Config::ConfigOptions) and an mt_scene_desc (the flat
// arrays Scene::Scene holds).  StartRender() returns at once (the render runs
// on the GPU and a host worker thread), WaitForRender() joins it and writes
// the image into the shared RenderBuffer, KillRender() may be called from any
// thread, GetStats()/IsDone() are safe while the render runs.  Failures throw
// std::runtime_error carrying the library's message, as the reference throws
// on setup errors; the hot path itself reports through the status codes.
#pragma once

#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../mitrace_gpu.h"

namespace mitrace {

// RenderBuffer (src/Tracer/RenderBuffer.hpp:11-35): W x H RGB floats, row-major.
class RenderBuffer {
   public:
    RenderBuffer(unsigned width, unsigned height)
        : width_(width), height_(height), pixels_(static_cast<size_t>(width) * height * 3, 0.0f)
    {
    }
    unsigned GetWidth() const { return width_; }
    unsigned GetHeight() const { return height_; }
    void GetPixel(unsigned x, unsigned y, float rgb[3]) const
    {
        if (x >= width_ || y >= height_) return;
        const float* p = &pixels_[(static_cast<size_t>(y) * width_ + x) * 3];
        rgb[0] = p[0];
        rgb[1] = p[1];
        rgb[2] = p[2];
    }
    void SetPixel(unsigned x, unsigned y, const float rgb[3])
    {
        if (x >= width_ || y >= height_) return;
        float* p = &pixels_[(static_cast<size_t>(y) * width_ + x) * 3];
        p[0] = rgb[0];
        p[1] = rgb[1];
        p[2] = rgb[2];
    }
    float* Data() { return pixels_.data(); }
    const float* Data() const { return pixels_.data(); }

    // GetPixelsRGB8 / SaveToFilePNG / SaveToFileHDR (RenderBuffer.cpp:37-84):
    // bytes are clamp(v * 255, 0, 255) truncated; the HDR file holds the floats.
    std::vector<uint8_t> GetPixelsRGB8() const
    {
        std::vector<uint8_t> out(pixels_.size());
        for (size_t i = 0; i < pixels_.size(); ++i) {
            float v = pixels_[i] * 255.0f;
            v = v < 0.0f ? 0.0f : (v > 255.0f ? 255.0f : v);
            out[i] = static_cast<uint8_t>(v);
        }
        return out;
    }
    void SaveToFilePNG(const std::string& filename) const
    {
        const std::vector<uint8_t> rgb = GetPixelsRGB8();
        if (mt_write_png(filename.c_str(), rgb.data(), width_, height_) != MT_OK)
            throw std::runtime_error("Failed to save image to file");
    }
    void SaveToFileHDR(const std::string& filename) const
    {
        if (mt_write_hdr(filename.c_str(), pixels_.data(), width_, height_) != MT_OK)
            throw std::runtime_error("Failed to save image to file");
    }

   private:
    unsigned width_, height_;
    std::vector<float> pixels_;
};

class Tracer {
   public:
    struct Stats {
        float progress;
        float timeElapsed;
        float estimatedTimeRemaining;
        size_t rays;
        size_t samples;
    };

    Tracer(std::shared_ptr<RenderBuffer> imageBuffer, const mt_scene_desc& scene, const mt_config& config)
        : imageBuffer_(std::move(imageBuffer))
    {
        if (!imageBuffer_) throw std::runtime_error("Tracer: null RenderBuffer");
        mt_config cfg = config;
        cfg.width = imageBuffer_->GetWidth();
        cfg.height = imageBuffer_->GetHeight();
        check(mt_create(&scene, &cfg, &handle_), "mt_create");
    }
    ~Tracer()
    {
        if (handle_) mt_destroy(handle_);
    }
    Tracer(const Tracer&) = delete;
    Tracer& operator=(const Tracer&) = delete;

    void StartRender() { check(mt_start(handle_), "mt_start"); }
    void WaitForRender() { check(mt_wait(handle_, imageBuffer_->Data()), "mt_wait"); }
    void KillRender() { mt_kill(handle_); }
    Stats GetStats() const
    {
        mt_stats s{};
        mt_get_stats(handle_, &s);
        return Stats{s.progress, s.time_elapsed, s.estimated_time_remaining, static_cast<size_t>(s.rays),
                     static_cast<size_t>(s.samples)};
    }
    bool IsDone() const { return mt_is_done(handle_) != 0; }

    mt_handle* Handle() const { return handle_; }

   private:
    static void check(mt_status s, const char* where)
    {
        if (s != MT_OK) throw std::runtime_error(std::string(where) + ": " + mt_last_error());
    }

    std::shared_ptr<RenderBuffer> imageBuffer_;
    mt_handle* handle_ = nullptr;
};

}  // namespace mitrace
