// mbcg_io.cu -- output of a case: VTI images (the reference's io/vtiWriter.cuh, plus a raw
// appended-binary encoding), an asynchronous writer that overlaps the device-to-host copy and the
// file writing with further steps, and a bit-exact checkpoint / restart format (no counterpart
// in the reference).  Declared in include/mbcg.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <condition_variable>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <deque>
#include <functional>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "mbcg_internal.h"

using namespace mbcg;

namespace {

int fail(int code, const std::string& msg) {
    set_last_error(msg);
    return code;
}
int cuda_fail(cudaError_t e, const char* what) {
    return fail(MBCG_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

const char* const kFieldNames[NF] = {"rhor", "rhob", "ux", "uy", "uz", "Pixx", "Pixy", "Piyy", "Piyz", "Pizz", "Pixz"};

std::vector<int> fields_of(uint32_t mask) {
    if (mask == 0) mask = MBCG_VTI_REFERENCE_FIELDS;
    std::vector<int> f;
    for (int i = 0; i < NF; ++i)
        if (mask & (1u << i)) f.push_back(i);
    return f;
}

// ---------------------------------------------------------------- VTI formatting
// The reference writes every value as std::scientific with precision 8 followed by a space, one
// x row per line (io/vtiWriter.cuh:60-85); "%.8e" of the value widened to double is the same text.
void format_rows(const float* v, long long nx, long long row0, long long row1, std::string& out) {
    char buf[32];
    out.clear();
    out.reserve(static_cast<size_t>((row1 - row0) * nx * 16));
    for (long long r = row0; r < row1; ++r) {
        const float* p = v + r * nx;
        for (long long x = 0; x < nx; ++x) {
            const int n = std::snprintf(buf, sizeof(buf), "%.8e ", static_cast<double>(p[x]));
            out.append(buf, static_cast<size_t>(n));
        }
        out.push_back('\n');
    }
}

std::string vti_head(const mbcg_params& p, bool raw) {
    std::string h = "<?xml version=\"1.0\"?>\n";
    h += raw ? "<VTKFile type=\"ImageData\" version=\"0.1\" byte_order=\"LittleEndian\" header_type=\"UInt64\">\n"
             : "<VTKFile type=\"ImageData\" version=\"0.1\" byte_order=\"LittleEndian\">\n";
    const std::string ext = "0 " + std::to_string(p.nx - 1) + " 0 " + std::to_string(p.ny - 1) + " 0 " +
                            std::to_string(p.nz - 1);
    h += "  <ImageData WholeExtent=\"" + ext + "\" Origin=\"0 0 0\" Spacing=\"1 1 1\">\n";
    h += "    <Piece Extent=\"" + ext + "\">\n";
    h += "      <PointData Scalars=\"rhor\">\n";
    return h;
}

// Writes fields (dense FP32, reference layout, one after another in `data`) to `path`.
int write_vti_file(const std::string& path, const mbcg_params& p, const std::vector<int>& fields, const float* data,
                   int format) {
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) return fail(MBCG_E_INVALID, "cannot open VTI file for writing: " + path);
    const long long n = static_cast<long long>(p.nx) * p.ny * p.nz;
    const long long rows = static_cast<long long>(p.ny) * p.nz;
    bool ok = true;
    const bool raw = format == MBCG_VTI_RAW;
    std::string head = vti_head(p, raw);
    if (raw) {
        unsigned long long off = 0;
        for (int fi : fields) {
            head += "        <DataArray type=\"Float32\" Name=\"" + std::string(kFieldNames[fi]) +
                    "\" format=\"appended\" offset=\"" + std::to_string(off) + "\"/>\n";
            off += 8 + static_cast<unsigned long long>(n) * 4;
        }
        head += "      </PointData>\n      <CellData>\n      </CellData>\n    </Piece>\n  </ImageData>\n";
        head += "  <AppendedData encoding=\"raw\">\n_";
        ok = std::fwrite(head.data(), 1, head.size(), f) == head.size();
        for (size_t k = 0; k < fields.size() && ok; ++k) {
            const unsigned long long nbytes = static_cast<unsigned long long>(n) * 4;
            ok = std::fwrite(&nbytes, 8, 1, f) == 1 &&
                 std::fwrite(data + k * n, 4, static_cast<size_t>(n), f) == static_cast<size_t>(n);
        }
        const char* tail = "\n  </AppendedData>\n</VTKFile>\n";
        ok = ok && std::fwrite(tail, 1, std::strlen(tail), f) == std::strlen(tail);
    } else {
        ok = std::fwrite(head.data(), 1, head.size(), f) == head.size();
        // rows are formatted by all host threads, written in order
        const unsigned hw = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
        for (size_t k = 0; k < fields.size() && ok; ++k) {
            const std::string open = "        <DataArray type=\"Float32\" Name=\"" + std::string(kFieldNames[fields[k]]) +
                                     "\" format=\"ascii\">\n";
            ok = std::fwrite(open.data(), 1, open.size(), f) == open.size();
            const float* v = data + k * n;
            const long long block = 4096; // rows per formatting task
            for (long long r0 = 0; r0 < rows && ok; r0 += block * hw) {
                std::vector<std::string> parts(hw);
                std::vector<std::thread> th;
                for (unsigned t = 0; t < hw; ++t) {
                    const long long a = r0 + t * block, b = std::min(rows, a + block);
                    if (a >= b) break;
                    th.emplace_back(format_rows, v, static_cast<long long>(p.nx), a, b, std::ref(parts[t]));
                }
                for (auto& t : th) t.join();
                for (const auto& s : parts)
                    if (ok && !s.empty()) ok = std::fwrite(s.data(), 1, s.size(), f) == s.size();
            }
            const char* close = "        </DataArray>\n";
            ok = ok && std::fwrite(close, 1, std::strlen(close), f) == std::strlen(close);
        }
        const char* tail = "      </PointData>\n      <CellData>\n      </CellData>\n    </Piece>\n  </ImageData>\n</VTKFile>\n";
        ok = ok && std::fwrite(tail, 1, std::strlen(tail), f) == std::strlen(tail);
    }
    ok = (std::fclose(f) == 0) && ok;
    return ok ? MBCG_OK : fail(MBCG_E_INVALID, "error while writing VTI file: " + path);
}

// ---------------------------------------------------------------- checkpoint
constexpr char kMagic[8] = {'M', 'B', 'C', 'G', 'C', 'K', 'P', '1'};

struct CheckpointHeader {
    char magic[8];
    uint32_t version;
    uint32_t header_bytes;
    mbcg_params params;
    int64_t steps;
    int32_t precision;
    int32_t nfields;
    int64_t nx, ny, nz;
    uint64_t payload_bytes;
    uint64_t payload_fnv1a;
};

uint64_t fnv1a(const unsigned char* p, size_t n, uint64_t h = 1469598103934665603ULL) {
    for (size_t i = 0; i < n; ++i) {
        h ^= p[i];
        h *= 1099511628211ULL;
    }
    return h;
}

} // namespace

// ---------------------------------------------------------------- asynchronous writer
struct mbcg_writer {
    struct Slot {
        float* dev = nullptr;
        float* host = nullptr;
        size_t cap = 0; // floats
        bool busy = false;
    };
    struct Job {
        int slot;
        cudaEvent_t copied;
        std::string path;
        mbcg_params p;
        std::vector<int> fields;
        int format;
    };
    int device = 0;
    cudaStream_t copy = nullptr;
    std::vector<Slot> slots;
    std::deque<Job> jobs;
    std::mutex mu;
    std::condition_variable cv;
    bool stop = false;
    int error = MBCG_OK;
    std::string error_msg;
    int pending = 0;
    std::thread worker;

    void run() {
        cudaSetDevice(device);
        std::unique_lock<std::mutex> lk(mu);
        for (;;) {
            cv.wait(lk, [&] { return stop || !jobs.empty(); });
            if (jobs.empty()) break;
            Job j = std::move(jobs.front());
            jobs.pop_front();
            lk.unlock();
            int rc = MBCG_OK;
            std::string msg;
            cudaError_t e = cudaEventSynchronize(j.copied);
            cudaEventDestroy(j.copied);
            if (e != cudaSuccess) {
                rc = MBCG_E_CUDA;
                msg = std::string("snapshot copy: ") + cudaGetErrorString(e);
            } else {
                rc = write_vti_file(j.path, j.p, j.fields, slots[j.slot].host, j.format);
                if (rc) msg = mbcg_last_error();
            }
            lk.lock();
            if (rc && error == MBCG_OK) {
                error = rc;
                error_msg = msg;
            }
            slots[j.slot].busy = false;
            pending -= 1;
            cv.notify_all();
        }
    }
};

extern "C" {

int mbcg_write_vti(mbcg_case* c, const char* path, uint32_t field_mask, int32_t format, mbcg_stream_t s) {
    if (!c || !path) return fail(MBCG_E_INVALID, "null argument");
    if (format != MBCG_VTI_ASCII && format != MBCG_VTI_RAW) return fail(MBCG_E_INVALID, "unknown VTI format");
    mbcg_params p;
    if (int rc = mbcg_case_params(c, &p)) return rc;
    const std::vector<int> fields = fields_of(field_mask);
    const size_t n = static_cast<size_t>(p.nx) * p.ny * p.nz;
    std::vector<float> host(n * fields.size());
    float* dev = nullptr;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(s);
    cudaError_t e = cudaMalloc(&dev, n * sizeof(float));
    for (size_t k = 0; k < fields.size() && e == cudaSuccess; ++k) {
        if (int rc = case_field_to_dense(c, fields[k], dev, st)) {
            cudaFree(dev);
            return rc;
        }
        e = cudaMemcpyAsync(host.data() + k * n, dev, n * sizeof(float), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    }
    if (dev) cudaFree(dev);
    if (e != cudaSuccess) return cuda_fail(e, "mbcg_write_vti");
    return write_vti_file(path, p, fields, host.data(), format);
}

int mbcg_writer_create(int32_t max_pending, mbcg_writer** out) {
    if (!out) return fail(MBCG_E_INVALID, "null output handle");
    *out = nullptr;
    if (max_pending <= 0) max_pending = 2;
    auto* w = new mbcg_writer();
    cudaError_t e = cudaGetDevice(&w->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&w->copy, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete w;
        return cuda_fail(e, "mbcg_writer_create");
    }
    w->slots.resize(max_pending);
    w->worker = std::thread([w] { w->run(); });
    *out = w;
    return MBCG_OK;
}

int mbcg_writer_snapshot(mbcg_writer* w, mbcg_case* c, const char* path, uint32_t field_mask, int32_t format,
                         mbcg_stream_t s) {
    if (!w || !c || !path) return fail(MBCG_E_INVALID, "null argument");
    if (format != MBCG_VTI_ASCII && format != MBCG_VTI_RAW) return fail(MBCG_E_INVALID, "unknown VTI format");
    mbcg_params p;
    if (int rc = mbcg_case_params(c, &p)) return rc;
    const std::vector<int> fields = fields_of(field_mask);
    const size_t n = static_cast<size_t>(p.nx) * p.ny * p.nz;
    const size_t need = n * fields.size();
    int slot = -1;
    {
        std::unique_lock<std::mutex> lk(w->mu);
        for (;;) {
            for (size_t i = 0; i < w->slots.size(); ++i)
                if (!w->slots[i].busy) {
                    slot = static_cast<int>(i);
                    break;
                }
            if (slot >= 0) break;
            w->cv.wait(lk); // every slot holds a snapshot not yet on disk: wait for one
        }
        w->slots[slot].busy = true;
        w->pending += 1;
    }
    mbcg_writer::Slot& sl = w->slots[slot];
    auto release = [&](int rc) {
        std::lock_guard<std::mutex> lk(w->mu);
        sl.busy = false;
        w->pending -= 1;
        w->cv.notify_all();
        return rc;
    };
    cudaStream_t st = reinterpret_cast<cudaStream_t>(s);
    if (sl.cap < need) {
        if (sl.dev) cudaFree(sl.dev);
        if (sl.host) cudaFreeHost(sl.host);
        sl.dev = nullptr;
        sl.host = nullptr;
        sl.cap = 0;
        cudaError_t e = cudaMalloc(&sl.dev, need * sizeof(float));
        if (e == cudaSuccess) e = cudaMallocHost(&sl.host, need * sizeof(float));
        if (e != cudaSuccess) return release(cuda_fail(e, "snapshot buffers"));
        sl.cap = need;
    }
    // on the case's stream: the snapshot of the current state (dense FP32), ordered before any
    // later step; then the copy to the host on the writer's stream, overlapping later steps
    for (size_t k = 0; k < fields.size(); ++k)
        if (int rc = case_field_to_dense(c, fields[k], sl.dev + k * n, st)) return release(rc);
    cudaEvent_t ready = nullptr, copied = nullptr;
    cudaError_t e = cudaEventCreateWithFlags(&ready, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&copied, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventRecord(ready, st);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(w->copy, ready, 0);
    if (e == cudaSuccess) e = cudaMemcpyAsync(sl.host, sl.dev, need * sizeof(float), cudaMemcpyDeviceToHost, w->copy);
    if (e == cudaSuccess) e = cudaEventRecord(copied, w->copy);
    if (ready) cudaEventDestroy(ready);
    if (e != cudaSuccess) {
        if (copied) cudaEventDestroy(copied);
        return release(cuda_fail(e, "snapshot"));
    }
    {
        std::lock_guard<std::mutex> lk(w->mu);
        w->jobs.push_back(mbcg_writer::Job{slot, copied, path, p, fields, format});
    }
    w->cv.notify_all();
    return MBCG_OK;
}

int mbcg_writer_flush(mbcg_writer* w) {
    if (!w) return fail(MBCG_E_INVALID, "null writer");
    std::unique_lock<std::mutex> lk(w->mu);
    w->cv.wait(lk, [&] { return w->pending == 0; });
    const int rc = w->error;
    if (rc) {
        set_last_error(w->error_msg);
        w->error = MBCG_OK;
    }
    return rc;
}

int mbcg_writer_destroy(mbcg_writer* w) {
    if (!w) return MBCG_OK;
    const int rc = mbcg_writer_flush(w);
    {
        std::lock_guard<std::mutex> lk(w->mu);
        w->stop = true;
    }
    w->cv.notify_all();
    w->worker.join();
    for (auto& sl : w->slots) {
        if (sl.dev) cudaFree(sl.dev);
        if (sl.host) cudaFreeHost(sl.host);
    }
    cudaStreamDestroy(w->copy);
    delete w;
    return rc;
}

// ---------------------------------------------------------------- checkpoint / restart
int mbcg_checkpoint_save(mbcg_case* c, const char* path, mbcg_stream_t s) {
    if (!c || !path) return fail(MBCG_E_INVALID, "null argument");
    CheckpointHeader h;
    std::memset(&h, 0, sizeof(h));
    std::memcpy(h.magic, kMagic, 8);
    h.version = 1;
    h.header_bytes = sizeof(h);
    if (int rc = mbcg_case_params(c, &h.params)) return rc;
    h.steps = mbcg_steps_done(c);
    h.precision = h.params.precision;
    h.nfields = NF;
    h.nx = h.params.nx;
    h.ny = h.params.ny;
    h.nz = h.params.nz;
    const size_t es = h.precision == MBCG_FP32 ? 4 : 2;
    const size_t n = static_cast<size_t>(h.nx) * h.ny * h.nz;
    h.payload_bytes = n * es * NF;
    std::vector<unsigned char> payload(h.payload_bytes);
    mbcg_moments a;
    if (int rc = mbcg_fields(c, &a, nullptr)) return rc;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(s);
    for (int i = 0; i < NF; ++i) {
        // the stored slots as they are, ghost frame included: a restart continues bit for bit
        cudaError_t e = cudaMemcpy2DAsync(payload.data() + i * n * es, h.nx * es, a.f[i], a.pitch * es, h.nx * es,
                                          static_cast<size_t>(h.ny) * h.nz, cudaMemcpyDeviceToHost, st);
        if (e != cudaSuccess) return cuda_fail(e, "checkpoint copy");
    }
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "checkpoint copy");
    h.payload_fnv1a = fnv1a(payload.data(), payload.size());
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(MBCG_E_INVALID, std::string("cannot open checkpoint for writing: ") + path);
    bool ok = std::fwrite(&h, sizeof(h), 1, f) == 1 && std::fwrite(payload.data(), 1, payload.size(), f) == payload.size();
    ok = (std::fclose(f) == 0) && ok;
    return ok ? MBCG_OK : fail(MBCG_E_INVALID, std::string("error while writing checkpoint: ") + path);
}

int mbcg_checkpoint_load(const char* path, mbcg_case** out) {
    if (!path || !out) return fail(MBCG_E_INVALID, "null argument");
    *out = nullptr;
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(MBCG_E_INVALID, std::string("cannot open checkpoint: ") + path);
    CheckpointHeader h;
    bool ok = std::fread(&h, sizeof(h), 1, f) == 1;
    if (!ok || std::memcmp(h.magic, kMagic, 8) != 0 || h.version != 1 || h.header_bytes != sizeof(h) ||
        h.nfields != NF || h.precision != h.params.precision || h.nx != h.params.nx || h.ny != h.params.ny ||
        h.nz != h.params.nz) {
        std::fclose(f);
        return fail(MBCG_E_INVALID, std::string("not an mbcg checkpoint of this version: ") + path);
    }
    const size_t es = h.precision == MBCG_FP32 ? 4 : 2;
    const size_t n = static_cast<size_t>(h.nx) * h.ny * h.nz;
    if (h.payload_bytes != n * es * NF) {
        std::fclose(f);
        return fail(MBCG_E_INVALID, "checkpoint payload size does not match its lattice");
    }
    std::vector<unsigned char> payload(h.payload_bytes);
    ok = std::fread(payload.data(), 1, payload.size(), f) == payload.size();
    std::fclose(f);
    if (!ok) return fail(MBCG_E_INVALID, "checkpoint truncated");
    if (fnv1a(payload.data(), payload.size()) != h.payload_fnv1a)
        return fail(MBCG_E_INVALID, "checkpoint checksum mismatch");
    mbcg_case* c = nullptr;
    if (int rc = mbcg_create(&h.params, &c)) return rc;
    mbcg_moments a;
    mbcg_fields(c, &a, nullptr);
    for (int i = 0; i < NF; ++i) {
        cudaError_t e = cudaMemcpy2D(a.f[i], a.pitch * es, payload.data() + i * n * es, h.nx * es, h.nx * es,
                                     static_cast<size_t>(h.ny) * h.nz, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            mbcg_destroy(c);
            return cuda_fail(e, "checkpoint restore");
        }
    }
    if (int rc = mirror_state(c, nullptr)) {
        mbcg_destroy(c);
        return rc;
    }
    if (cudaError_t e = cudaDeviceSynchronize()) {
        mbcg_destroy(c);
        return cuda_fail(e, "checkpoint restore");
    }
    case_set_steps(c, h.steps);
    *out = c;
    return MBCG_OK;
}

} // extern "C"
