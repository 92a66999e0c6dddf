// Shim for the missing LiteImage header (HydraCore3): the Image2D container,
// its sampler description and the combined image-sampler interface, as the
// reference's renderer and differentiable renderer use them.  For compiling
// the reference in place (oracle pinning only).  sample() is a texel-centred
// bilinear filter with clamp-to-edge addressing (the library's own filter is
// not in the reference tree; at texel centres, where the pinned fixtures
// sample, every bilinear filter returns the texel itself).  SaveImage writes
// nothing.
#pragma once
#include <cstdint>
#include <memory>
#include <vector>
#include "LiteMath.h"

namespace LiteImage {
struct Sampler {
  enum class AddressMode { WRAP, MIRROR, CLAMP, BORDER, MIRROR_ONCE };
  enum class Filter { NEAREST, LINEAR, CUBIC };
  AddressMode addressU = AddressMode::CLAMP, addressV = AddressMode::CLAMP, addressW = AddressMode::CLAMP;
  LiteMath::float4 borderColor = LiteMath::float4(0, 0, 0, 0);
  Filter filter = Filter::NEAREST;
};

template <typename T>
struct Image2D {
  Image2D() = default;
  Image2D(unsigned w, unsigned h) : m_w(w), m_h(h), m_data(size_t(w) * h) {}
  Image2D(unsigned w, unsigned h, const T &v) : m_w(w), m_h(h), m_data(size_t(w) * h, v) {}
  unsigned width() const { return m_w; }
  unsigned height() const { return m_h; }
  T *data() { return m_data.data(); }
  const T *data() const { return m_data.data(); }
  void clear(const T &v) { std::fill(m_data.begin(), m_data.end(), v); }
  T &operator[](LiteMath::uint2 p) { return m_data[size_t(p.y) * m_w + p.x]; }
  const T &operator[](LiteMath::uint2 p) const { return m_data[size_t(p.y) * m_w + p.x]; }
  T texel(int x, int y) const {
    x = x < 0 ? 0 : (x >= int(m_w) ? int(m_w) - 1 : x);
    y = y < 0 ? 0 : (y >= int(m_h) ? int(m_h) - 1 : y);
    return m_data[size_t(y) * m_w + x];
  }
  T sample(const Sampler &s, LiteMath::float2 uv) const {
    const float fx = uv.x * float(m_w) - 0.5f, fy = uv.y * float(m_h) - 0.5f;
    if (s.filter == Sampler::Filter::NEAREST) return texel(int(std::floor(fx + 0.5f)), int(std::floor(fy + 0.5f)));
    const float x0 = std::floor(fx), y0 = std::floor(fy);
    const float ax = fx - x0, ay = fy - y0;
    const int ix = int(x0), iy = int(y0);
    return (texel(ix, iy) * (1.0f - ax) + texel(ix + 1, iy) * ax) * (1.0f - ay) +
           (texel(ix, iy + 1) * (1.0f - ax) + texel(ix + 1, iy + 1) * ax) * ay;
  }
  unsigned m_w = 0, m_h = 0;
  std::vector<T> m_data;
};

template <typename T>
static inline bool SaveImage(const char *, const Image2D<T> &, float = 2.2f) { return true; }

struct ICombinedImageSampler {
  virtual ~ICombinedImageSampler() {}
  virtual LiteMath::float4 sample(LiteMath::float2 uv) const = 0;
};

template <typename T>
struct CombinedImageSampler : ICombinedImageSampler {
  std::shared_ptr<Image2D<T>> image;
  Sampler sampler;
  LiteMath::float4 sample(LiteMath::float2 uv) const override { return image->sample(sampler, uv); }
};

template <typename T>
static inline std::shared_ptr<ICombinedImageSampler> MakeCombinedTexture2D(std::shared_ptr<Image2D<T>> img,
                                                                          Sampler s) {
  auto p = std::make_shared<CombinedImageSampler<T>>();
  p->image = img;
  p->sampler = s;
  return p;
}
}  // namespace LiteImage
