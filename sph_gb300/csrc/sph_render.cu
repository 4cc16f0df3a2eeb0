// sph_render.cu -- the render rank's liquid-surface image as compute
// kernels into device buffers (no graphics API): the four passes of
// draw_liquid (liquid_gl.c:305-447) at the reduced texture resolution
// (screen / 2, liquid_gl.c:43-48) and the composite at screen resolution.
//
//   1 k_splat      metaball point sprites (shaders/liquid_particle.frag:10-20):
//                  intensity 1 - 3 r^2 for r^2 <= 0.34 (r in units of the
//                  sprite radius), additive blending into an 8-bit alpha
//                  texture (liquid_gl.c:318-343, 106): every fragment adds
//                  round(255 i), the sum saturates at 255.  Integer atomics
//                  make the result independent of the drawing order.
//   2 k_blur<V>    15-tap Gaussian along y, then along x
//                  (shaders/vert_blur.vert:12-26, horz_blur.vert,
//                  blur.frag:12-29): taps at +-0.004 k texture units,
//                  bilinear filtering with clamp to edge (liquid_gl.c:107-110),
//                  each pass stored back to 8 bits.
//   3 k_composite  shaders/render_liquid_texture.frag:11-17 at screen size:
//                  alpha a (bilinear), discard below 0.1, colour
//                  (w, w, 1) with w = smoothstep(-0.15, -0.1, -a) blended
//                  with alpha 0.75 smoothstep(0.1, 0.11, a) over a black
//                  background (liquid_gl.c:436-444).
// The blur passes' texture-coordinate flips (liquid_gl.c:146-160 and
// render_liquid_texture.vert) cancel in pairs and the kernel is symmetric,
// so images are kept bottom row first until the final file order.
#include <cmath>

#include "sph_internal.h"

namespace sph {
namespace render {

// Gaussian taps of blur.frag (centre, then +-1 .. +-7 in steps of 0.004).
__constant__ float kTap[8] = {0.159576912161f, 0.147308056121f, 0.115876621105f,
                              0.0776744219933f, 0.0443683338718f, 0.0215963866053f,
                              0.00895781211794f, 0.0044299121055113265f};

// Sprite geometry: points are the packed shorts / SHRT_MAX in [-1, 1]
// (renderer.c:333-337); the sprite diameter is 0.020 of the screen width
// (renderer.c:224), divided by the texture reduction (liquid_gl.c:77).
__global__ void k_splat(int n, const short2 *__restrict__ coords, int w, int h, float radius,
                        unsigned *__restrict__ acc)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const short2 c = coords[i];
    const float px = (float)c.x / 32767.0f, py = (float)c.y / 32767.0f;
    const float cx = (px + 1.0f) * 0.5f * (float)w, cy = (py + 1.0f) * 0.5f * (float)h;
    const float reach = 0.5831f * radius + 1.0f;  // sqrt(0.34) = 0.5831
    const int x0 = max(0, (int)floorf(cx - reach)), x1 = min(w - 1, (int)ceilf(cx + reach));
    const int y0 = max(0, (int)floorf(cy - reach)), y1 = min(h - 1, (int)ceilf(cy + reach));
    const float inv = 1.0f / radius;
    for (int y = y0; y <= y1; ++y) {
        const float dy = ((float)y + 0.5f - cy) * inv;
        for (int x = x0; x <= x1; ++x) {
            const float dx = ((float)x + 0.5f - cx) * inv;
            const float r2 = dx * dx + dy * dy;
            if (r2 > 0.34f) continue;
            const int v = __float2int_rn((1.0f - 3.0f * r2) * 255.0f);
            if (v > 0) atomicAdd(acc + (size_t)y * w + x, (unsigned)v);
        }
    }
}

__global__ void k_saturate(int m, const unsigned *__restrict__ acc, unsigned char *__restrict__ a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) a[i] = (unsigned char)min(acc[i], 255u);
}

// Bilinear sample of an 8-bit texture along one axis at texel coordinate t
// (texel centres at integers), clamped to the edge.
__device__ __forceinline__ float lerp_axis(const unsigned char *__restrict__ row, int stride,
                                           int len, float t)
{
    const float f = floorf(t);
    const int i0 = (int)f;
    const float a = t - f;
    const int j0 = min(max(i0, 0), len - 1), j1 = min(max(i0 + 1, 0), len - 1);
    return (1.0f - a) * (float)row[(size_t)j0 * stride] + a * (float)row[(size_t)j1 * stride];
}

// One blur pass: VERTICAL along y (offsets in units of the texture height),
// else along x.  Output stored to 8 bits.
template <bool VERTICAL>
__global__ void k_blur(int w, int h, const unsigned char *__restrict__ in,
                       unsigned char *__restrict__ out)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x >= w || y >= h) return;
    const int len = VERTICAL ? h : w;
    const int pos = VERTICAL ? y : x;
    const unsigned char *line = VERTICAL ? in + x : in + (size_t)y * w;
    const int stride = VERTICAL ? w : 1;
    float s = kTap[0] * (float)line[(size_t)pos * stride];
#pragma unroll
    for (int k = 1; k <= 7; ++k) {
        const float o = 0.004f * (float)k * (float)len;
        s += kTap[k] * (lerp_axis(line, stride, len, (float)pos - o) +
                        lerp_axis(line, stride, len, (float)pos + o));
    }
    out[(size_t)y * w + x] = (unsigned char)min(255, max(0, __float2int_rn(s)));
}

__device__ __forceinline__ float smoothstep(float e0, float e1, float x)
{
    const float t = fminf(fmaxf((x - e0) / (e1 - e0), 0.0f), 1.0f);
    return t * t * (3.0f - 2.0f * t);
}

// Screen pixel (X, Y) (Y = 0 at the bottom) -> RGB8, written top row first.
__global__ void k_composite(int W, int H, int w, int h, const unsigned char *__restrict__ a,
                            unsigned char *__restrict__ rgb)
{
    const int X = blockIdx.x * blockDim.x + threadIdx.x;
    const int Y = blockIdx.y;
    if (X >= W || Y >= H) return;
    const float u = ((float)X + 0.5f) / (float)W * (float)w - 0.5f;
    const float v = ((float)Y + 0.5f) / (float)H * (float)h - 0.5f;
    const float fu = floorf(u), fv = floorf(v);
    const int i0 = (int)fu, j0 = (int)fv;
    const float au = u - fu, av = v - fv;
    const int ia = min(max(i0, 0), w - 1), ib = min(max(i0 + 1, 0), w - 1);
    const int ja = min(max(j0, 0), h - 1), jb = min(max(j0 + 1, 0), h - 1);
    const float s00 = a[(size_t)ja * w + ia], s01 = a[(size_t)ja * w + ib];
    const float s10 = a[(size_t)jb * w + ia], s11 = a[(size_t)jb * w + ib];
    const float alpha = ((1.0f - av) * ((1.0f - au) * s00 + au * s01) +
                         av * ((1.0f - au) * s10 + au * s11)) / 255.0f;
    float r = 0.0f, g = 0.0f, b = 0.0f;
    if (alpha >= 0.1f) {
        const float o = 0.75f * smoothstep(0.1f, 0.11f, alpha);
        const float white = smoothstep(-0.15f, -0.1f, -alpha);
        r = white * o;
        g = white * o;
        b = o;
    }
    unsigned char *p = rgb + ((size_t)(H - 1 - Y) * W + X) * 3;
    p[0] = (unsigned char)__float2int_rn(r * 255.0f);
    p[1] = (unsigned char)__float2int_rn(g * 255.0f);
    p[2] = (unsigned char)__float2int_rn(b * 255.0f);
}

}  // namespace render

int launch_pack(sph_cuda *h, short2 *out);

// The whole image from device coordinates; scratch holds the reduced
// textures.  alpha_out (optional, device) receives the blurred reduced alpha.
static int render_device(cudaStream_t st, const short2 *coords, int n, int W, int H,
                         unsigned char *d_rgb, unsigned char *scratch, unsigned char *alpha_out)
{
    using namespace render;
    const int w = W / 2, h = H / 2;
    const size_t m = (size_t)w * h;
    unsigned *acc = reinterpret_cast<unsigned *>(scratch);
    unsigned char *t0 = scratch + ((m * 4 + 255) & ~(size_t)255);
    unsigned char *t1 = t0 + ((m + 255) & ~(size_t)255);
    int rc = cuda_fail(cudaMemsetAsync(acc, 0, m * 4, st), "clear");
    if (rc) return rc;
    const float radius = 0.5f * ((float)W * 0.020f / 2.0f);
    if (n > 0) k_splat<<<(n + 255) / 256, 256, 0, st>>>(n, coords, w, h, radius, acc);
    k_saturate<<<(int)((m + 255) / 256), 256, 0, st>>>((int)m, acc, t0);
    const dim3 rows((w + 255) / 256, h);
    k_blur<true><<<rows, 256, 0, st>>>(w, h, t0, t1);
    k_blur<false><<<rows, 256, 0, st>>>(w, h, t1, t0);
    if (alpha_out) cudaMemcpyAsync(alpha_out, t0, m, cudaMemcpyDeviceToDevice, st);
    k_composite<<<dim3((W + 255) / 256, H), 256, 0, st>>>(W, H, w, h, t0, d_rgb);
    return cuda_fail(cudaGetLastError(), "render");
}

static size_t render_scratch(int W, int H)
{
    const size_t m = (size_t)(W / 2) * (H / 2);
    return ((m * 4 + 255) & ~(size_t)255) + 2 * ((m + 255) & ~(size_t)255);
}

static int check_size(int W, int H)
{
    if (W < 2 || H < 2 || W > 16384 || H > 16384) {
        set_error("image size %d x %d outside [2, 16384]", W, H);
        return SPH_ERR_INVALID;
    }
    return SPH_OK;
}

}  // namespace sph

using namespace sph;

extern "C" {

int sph_render_liquid(const short *coords, int n, int width, int height, unsigned char *rgb,
                      unsigned char *alpha)
{
    if ((!coords && n > 0) || n < 0 || !rgb) {
        set_error("sph_render_liquid: bad arguments");
        return SPH_ERR_INVALID;
    }
    int rc = check_size(width, height);
    if (rc) return rc;
    const size_t img = (size_t)width * height * 3, m = (size_t)(width / 2) * (height / 2);
    const size_t cb = (((size_t)n * 4) + 255) & ~(size_t)255;
    unsigned char *buf = nullptr;
    cudaStream_t st = nullptr;
    rc = cuda_fail(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "stream");
    if (rc) return rc;
    const size_t total = cb + ((img + 255) & ~(size_t)255) + ((m + 255) & ~(size_t)255) +
                         render_scratch(width, height);
    rc = cuda_fail(cudaMalloc(&buf, total), "cudaMalloc");
    if (!rc) {
        short2 *d_coords = reinterpret_cast<short2 *>(buf);
        unsigned char *d_rgb = buf + cb;
        unsigned char *d_alpha = d_rgb + ((img + 255) & ~(size_t)255);
        unsigned char *scratch = d_alpha + ((m + 255) & ~(size_t)255);
        if (n > 0)
            rc = cuda_fail(cudaMemcpyAsync(d_coords, coords, (size_t)n * 4, cudaMemcpyHostToDevice, st),
                           "coords");
        if (!rc) rc = render_device(st, d_coords, n, width, height, d_rgb, scratch, d_alpha);
        if (!rc) rc = cuda_fail(cudaMemcpyAsync(rgb, d_rgb, img, cudaMemcpyDeviceToHost, st), "image");
        if (!rc && alpha)
            rc = cuda_fail(cudaMemcpyAsync(alpha, d_alpha, m, cudaMemcpyDeviceToHost, st), "alpha");
        if (!rc) rc = cuda_fail(cudaStreamSynchronize(st), "sync");
    }
    cudaStreamSynchronize(st);
    if (buf) cudaFree(buf);
    cudaStreamDestroy(st);
    return rc;
}

int sph_cuda_render_liquid(sph_cuda_t *h, int width, int height, unsigned char *rgb,
                           unsigned char *alpha)
{
    if (!h || !rgb) {
        set_error("sph_cuda_render_liquid: null argument");
        return SPH_ERR_INVALID;
    }
    int rc = check_size(width, height);
    if (rc) return rc;
    const int n = h->n;
    const size_t img = (size_t)width * height * 3, m = (size_t)(width / 2) * (height / 2);
    const size_t cb = (((size_t)n * 4) + 255) & ~(size_t)255;
    const size_t ib = (img + 255) & ~(size_t)255, ab = (m + 255) & ~(size_t)255;
    rc = ensure_scratch(h, cb + ib + ab + render_scratch(width, height) + 256);
    if (rc) return rc;
    unsigned char *base = (unsigned char *)h->d_scratch;
    short2 *d_coords = reinterpret_cast<short2 *>(base);
    unsigned char *d_rgb = base + cb, *d_alpha = d_rgb + ib, *scratch = d_alpha + ab;
    if (n > 0) {
        rc = launch_pack(h, d_coords);
        if (rc) return rc;
    }
    rc = render_device(h->stream, d_coords, n, width, height, d_rgb, scratch, d_alpha);
    if (!rc) rc = cuda_fail(cudaMemcpyAsync(rgb, d_rgb, img, cudaMemcpyDeviceToHost, h->stream), "image");
    if (!rc && alpha)
        rc = cuda_fail(cudaMemcpyAsync(alpha, d_alpha, m, cudaMemcpyDeviceToHost, h->stream), "alpha");
    if (!rc) rc = cuda_fail(cudaStreamSynchronize(h->stream), "sync");
    return rc;
}

}  // extern "C"
