// The FacesNMF data set: PGM loader and CSV writer
// (src/examples/FacesNMF/FacesNMFDlg.cpp:309-472 and 913-936).
//
// Loading: the files are read on the host (many threads), their pixel bytes
// packed into one pinned buffer and copied to the device in one transfer
// (a quarter of the bytes of the FP32 matrix), then one CTA per image builds
// the 256-bin histogram in shared memory, its cumulative counts and the
// equalisation table, and writes the image's column of V (pixels x images,
// column-major FP32) straight into device memory, where an NMF job can take it
// without another copy.  The arithmetic is the reference's, in float:
//   equalised:  (cum[p] - cdfmin) / (pixels - cdfmin), cdfmin = first nonzero cum
//   plain:      p / 255
// with IEEE round-to-nearest division, so the device result equals a CPU
// float restatement bit for bit.
//
// The reference reads the pixel block with istream::read right after
// `>> maxGrayValue` (:434-443), i.e. starting AT the single whitespace byte
// that ends the header: its pixel 0 is that byte ('\n' in the data set's
// files) and the image's last pixel is never read.  reference_offset = 1
// keeps that (the drop-in default, identical V); 0 reads the pixels where the
// PGM format puts them.
//
// Writing: Save() prints every column of a matrix as one line of
// comma-separated values in fixed notation with 20 decimals (PRECISION,
// src/examples/FacesNMF/Definitions.h:31).  Formatting is split by columns
// over host threads and the pieces are written in order.
#include <errno.h>
#include <stdio.h>
#include <string.h>
#include <sys/stat.h>

#include <algorithm>
#include <string>
#include <thread>
#include <vector>

#include "common.cuh"
#include "engine.h"

namespace gpunmf {

__global__ void __launch_bounds__(256) faces_to_v_kernel(const unsigned char *__restrict__ bytes, int pixels,
                                                         int count, int equalize,
                                                         const unsigned char *__restrict__ ok,
                                                         float *__restrict__ V, long long ldv) {
    __shared__ unsigned int cum[256];
    __shared__ float lut[256];
    __shared__ int first;
    const int t = threadIdx.x;
    for (int img = blockIdx.x; img < count; img += gridDim.x) {
        const unsigned char *px = bytes + (long long)img * pixels;
        float *col = V + (long long)img * ldv;
        if (!ok[img]) {  // an image that failed to load: a zero column
            for (int b = t; b < pixels; b += blockDim.x) col[b] = 0.f;
            continue;
        }
        if (equalize) {
            cum[t] = 0;
            __syncthreads();
            for (int b = t; b < pixels; b += blockDim.x) atomicAdd(&cum[px[b]], 1u);
            __syncthreads();
            // inclusive prefix sum over the 256 bins: warp 0, eight bins per lane
            if (t < 32) {
                unsigned int v[8], run = 0;
#pragma unroll
                for (int q = 0; q < 8; q++) {
                    run += cum[t * 8 + q];
                    v[q] = run;
                }
                unsigned int off = run;
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    const unsigned int o = __shfl_up_sync(0xffffffffu, off, d);
                    if (t >= d) off += o;
                }
                off -= run;  // exclusive offset of this lane's eight bins
#pragma unroll
                for (int q = 0; q < 8; q++) cum[t * 8 + q] = v[q] + off;
            }
            __syncthreads();
            // the first nonzero cumulative count (the counts are nondecreasing, so exactly one thread matches)
            if (cum[t] != 0 && (t == 0 || cum[t - 1] == 0)) first = t;
            __syncthreads();
            const float cdfmin = (float)cum[first];
            lut[t] = t >= first ? __fdiv_rn((float)cum[t] - cdfmin, (float)pixels - cdfmin) : 0.f;
        } else {
            lut[t] = __fdiv_rn((float)t, 255.0f);
        }
        __syncthreads();
        for (int b = t; b < pixels; b += blockDim.x) col[b] = lut[px[b]];
        __syncthreads();
    }
}

// ------------------------------------------------------------------------
// PGM header reading with the semantics of istream's >> (skip whitespace,
// then a token / a decimal integer)
// ------------------------------------------------------------------------
namespace {

bool is_space(int c) { return c == ' ' || c == '\n' || c == '\r' || c == '\t' || c == '\v' || c == '\f'; }

struct Reader {
    const std::vector<unsigned char> &buf;
    size_t pos = 0;
    void skip_ws() {
        while (pos < buf.size() && is_space(buf[pos])) pos++;
    }
    bool token(std::string &s) {
        skip_ws();
        s.clear();
        while (pos < buf.size() && !is_space(buf[pos])) s.push_back((char)buf[pos++]);
        return !s.empty();
    }
    bool integer(int &v) {
        skip_ws();
        size_t p = pos;
        bool neg = false;
        if (p < buf.size() && (buf[p] == '+' || buf[p] == '-')) neg = buf[p++] == '-';
        long long x = 0;
        size_t d0 = p;
        while (p < buf.size() && buf[p] >= '0' && buf[p] <= '9' && x < (1LL << 31)) x = x * 10 + (buf[p++] - '0');
        if (p == d0 || x >= (1LL << 31)) return false;
        pos = p;
        v = (int)(neg ? -x : x);
        return true;
    }
};

bool read_file(const std::string &path, std::vector<unsigned char> &out) {
    FILE *f = fopen(path.c_str(), "rb");
    if (!f) return false;
    out.clear();
    unsigned char chunk[65536];
    size_t k;
    while ((k = fread(chunk, 1, sizeof(chunk), f)) > 0) out.insert(out.end(), chunk, chunk + k);
    const bool ok = !ferror(f);
    fclose(f);
    return ok;
}

std::string face_path(const char *folder, int number) {
    char name[32];
    snprintf(name, sizeof(name), "face%05d.pgm", number);
    std::string p(folder);
    if (!p.empty() && p.back() != '/') p.push_back('/');
    return p + name;
}

bool file_exists(const std::string &path) {
    struct stat st;
    return stat(path.c_str(), &st) == 0 && S_ISREG(st.st_mode);
}

// LoadImage (:409-472) up to the pixel block; returns an error text or "" and fills `pixels_out`
std::string parse_image(const std::string &path, int width, int height, int reference_offset,
                        unsigned char *pixels_out) {
    std::vector<unsigned char> buf;
    if (!read_file(path, buf)) return "cannot read " + path;
    Reader rd{buf};
    std::string magic;
    int w = 0, h = 0, maxval = 0;
    if (!rd.token(magic) || magic != "P5") return "Invalid image format: " + path;
    if (!rd.integer(w) || !rd.integer(h) || w != width || h != height) return "Incorrect image size: " + path;
    if (!rd.integer(maxval) || maxval != 255) return "Check max gray value: " + path;
    size_t start = rd.pos;                                         // the reference reads from here
    if (!reference_offset && start < buf.size() && is_space(buf[start])) start++;  // PGM: one whitespace byte
    const size_t pixels = (size_t)width * height;
    if (buf.size() < start + pixels) return "image data too short: " + path;
    memcpy(pixels_out, buf.data() + start, pixels);
    return "";
}

}  // namespace

static gpunmf_status faces_load_impl(const char *folder, int count, int width, int height, int equalize,
                                     int reference_offset, float *V, bool v_on_device, cudaStream_t stream,
                                     int *failed) {
    if (!folder || !V || count <= 0 || width <= 0 || height <= 0 || (long long)width * height > (1 << 30)) {
        set_error("invalid faces load arguments");
        return GPUNMF_ERR_INVALID;
    }
    int devs = 0;
    if (cudaGetDeviceCount(&devs) != cudaSuccess || devs == 0) {
        cudaGetLastError();
        set_error("no CUDA device available");
        return GPUNMF_ERR_NO_DEVICE;
    }
    const size_t pixels = (size_t)width * height;
    const size_t total = pixels * (size_t)count;
    unsigned char *stage = nullptr;
    if (cudaHostAlloc((void **)&stage, total + count, cudaHostAllocDefault) != cudaSuccess) {
        cudaGetLastError();
        set_error("pinned staging allocation of %zu bytes failed", total + count);
        return GPUNMF_ERR_NOMEM;
    }
    unsigned char *okflags = stage + total;
    // read the files on several host threads, each a contiguous range of images
    std::vector<std::string> errors(count);
    const int nthreads = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    std::vector<std::thread> pool;
    for (int th = 0; th < nthreads; th++) {
        pool.emplace_back([&, th] {
            for (int i = th; i < count; i += nthreads) {
                errors[i] = parse_image(face_path(folder, i + 1), width, height, reference_offset,
                                        stage + pixels * (size_t)i);
                okflags[i] = errors[i].empty() ? 1 : 0;
                if (!okflags[i]) memset(stage + pixels * (size_t)i, 0, pixels);
            }
        });
    }
    for (auto &t : pool) t.join();
    int nfail = 0;
    std::string first_error;
    for (int i = 0; i < count; i++)
        if (!okflags[i]) {
            if (nfail++ == 0) first_error = errors[i];
        }
    if (failed) *failed = nfail;

    cudaStream_t s = stream;
    bool own = false;
    gpunmf_status st = GPUNMF_OK;
    unsigned char *d_bytes = nullptr;
    float *dV = v_on_device ? V : nullptr;
    cudaError_t e = cudaSuccess;
    if (!s) {
        e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
        own = e == cudaSuccess;
    }
    if (e == cudaSuccess) e = cudaMallocAsync((void **)&d_bytes, total + count, s);
    if (e == cudaSuccess && !v_on_device) e = cudaMallocAsync((void **)&dV, total * sizeof(float), s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_bytes, stage, total + count, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        const int grid = std::min(count, 8 * kNumSMsGB300);
        faces_to_v_kernel<<<grid, 256, 0, s>>>(d_bytes, (int)pixels, count, equalize ? 1 : 0, d_bytes + total, dV,
                                                 (long long)pixels);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && !v_on_device)
        e = cudaMemcpyAsync(V, dV, total * sizeof(float), cudaMemcpyDeviceToHost, s);
    if (d_bytes) cudaFreeAsync(d_bytes, s);
    if (dV && !v_on_device) cudaFreeAsync(dV, s);
    cudaError_t e2 = cudaStreamSynchronize(s);  // the staging buffer is read by the copy
    if (e == cudaSuccess) e = e2;
    if (own) cudaStreamDestroy(s);
    cudaFreeHost(stage);
    if (e != cudaSuccess) {
        set_error("faces load: %s", cudaGetErrorString(e));
        cudaGetLastError();
        st = GPUNMF_ERR_CUDA;
    } else if (nfail > 0) {
        set_error("%d image(s) failed to load (their columns are zero); first: %s", nfail, first_error.c_str());
        st = GPUNMF_ERR_INVALID;
    }
    return st;
}

// ------------------------------------------------------------------------
// CSV
// ------------------------------------------------------------------------
static gpunmf_status save_csv_impl(const char *path, const float *M, int rows, int cols) {
    if (!path || (!M && rows * (long long)cols > 0) || rows < 0 || cols < 0) {
        set_error("invalid CSV arguments");
        return GPUNMF_ERR_INVALID;
    }
    FILE *f = fopen(path, "wb");
    if (!f) {
        set_error("cannot open %s: %s", path, strerror(errno));
        return GPUNMF_ERR_INVALID;
    }
    const int nthreads = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    const int per_pass = 64 * nthreads;  // columns formatted per pass, in memory at once
    std::vector<std::string> text(per_pass);
    bool ok = true;
    for (int c0 = 0; c0 < cols && ok; c0 += per_pass) {
        const int c1 = std::min(cols, c0 + per_pass);
        std::vector<std::thread> pool;
        for (int th = 0; th < nthreads; th++) {
            pool.emplace_back([&, th] {
                char num[512];
                for (int c = c0 + th; c < c1; c += nthreads) {
                    std::string &out = text[c - c0];
                    out.clear();
                    const float *col = M + (size_t)c * rows;
                    for (int rr = 0; rr < rows; rr++) {
                        const int k = snprintf(num, sizeof(num), "%.20f", (double)col[rr]);
                        out.append(num, (size_t)std::max(0, std::min(k, (int)sizeof(num) - 1)));
                        if (rr + 1 < rows) out.push_back(',');
                    }
                    out.push_back('\n');
                }
            });
        }
        for (auto &t : pool) t.join();
        for (int c = c0; c < c1 && ok; c++) ok = fwrite(text[c - c0].data(), 1, text[c - c0].size(), f) == text[c - c0].size();
    }
    if (fclose(f) != 0) ok = false;
    if (!ok) {
        set_error("write to %s failed", path);
        return GPUNMF_ERR_INVALID;
    }
    return GPUNMF_OK;
}

}  // namespace gpunmf

using namespace gpunmf;

extern "C" {

gpunmf_status gpunmf_faces_scan(const char *folder, int *count, int *width, int *height) {
    if (!folder || !count || !width || !height) {
        set_error("invalid faces scan arguments");
        return GPUNMF_ERR_INVALID;
    }
    *count = 0;
    std::vector<unsigned char> buf;
    const std::string first = face_path(folder, 1);
    if (!read_file(first, buf)) {
        set_error("Error loading images: cannot read %s", first.c_str());
        return GPUNMF_ERR_INVALID;
    }
    Reader rd{buf};
    std::string magic;
    if (!rd.token(magic) || magic != "P5") {
        set_error("Invalid image format: %s", first.c_str());
        return GPUNMF_ERR_INVALID;
    }
    if (!rd.integer(*width) || !rd.integer(*height) || *width <= 0 || *height <= 0) {
        set_error("Error loading images: bad size in %s", first.c_str());
        return GPUNMF_ERR_INVALID;
    }
    // FolderHasImages (:331-346): steps of 1024 halved on every miss, down to 1
    int n = 0, inc = 1024;
    for (;;) {
        if (!file_exists(face_path(folder, n + inc))) {
            if (inc == 1) break;
            inc >>= 1;
        } else {
            n += inc;
        }
    }
    *count = n;
    return GPUNMF_OK;
}

gpunmf_status gpunmf_faces_load(const char *folder, int count, int width, int height, int equalize,
                                int reference_offset, float *V, int *failed) {
    return faces_load_impl(folder, count, width, height, equalize, reference_offset, V, false, nullptr, failed);
}

gpunmf_status gpunmf_faces_load_device(const char *folder, int count, int width, int height, int equalize,
                                       int reference_offset, float *dV, void *stream, int *failed) {
    return faces_load_impl(folder, count, width, height, equalize, reference_offset, dV, true,
                           (cudaStream_t)stream, failed);
}

gpunmf_status gpunmf_save_csv(const char *path, const float *M, int rows, int cols) {
    return save_csv_impl(path, M, rows, cols);
}

gpunmf_status gpunmf_save_csv_device(const char *path, const float *dM, int rows, int cols, void *stream) {
    if (!dM || rows < 0 || cols < 0) {
        set_error("invalid CSV arguments");
        return GPUNMF_ERR_INVALID;
    }
    const size_t count = (size_t)rows * cols;
    float *h = nullptr;
    if (count && cudaHostAlloc((void **)&h, count * sizeof(float), cudaHostAllocDefault) != cudaSuccess) {
        cudaGetLastError();
        set_error("pinned allocation failed");
        return GPUNMF_ERR_NOMEM;
    }
    cudaError_t e = cudaSuccess;
    if (count) e = cudaMemcpyAsync(h, dM, count * sizeof(float), cudaMemcpyDeviceToHost, (cudaStream_t)stream);
    if (e == cudaSuccess && count) e = cudaStreamSynchronize((cudaStream_t)stream);
    gpunmf_status st = GPUNMF_OK;
    if (e != cudaSuccess) {
        set_error("CSV read-back: %s", cudaGetErrorString(e));
        st = GPUNMF_ERR_CUDA;
    } else {
        st = save_csv_impl(path, h, rows, cols);
    }
    if (h) cudaFreeHost(h);
    return st;
}

}  // extern "C"
