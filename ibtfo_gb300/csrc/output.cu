// Output: VTK files of a case's state, and checkpoints to restart from.
//
// VTK: the legacy structured-points file the reference's WriteData writes
// (Src/Utils/WriteData.cpp:30-120): the interior cells as points, fields
// density / x-vel / y-vel / pressure, non-fluid cells marked -1 (density) and
// -100 (velocities, pressure), density floored at 1e-6, the time as field
// data; ASCII with the reference's "%f" values, or big-endian binary floats
// (an 8192x4096 grid in ASCII would take gigabytes).  The fields are derived
// on the GPU; only the four float planes cross to the host.
//
// Checkpoints (save/load in capi.cu) keep the state buffers' raw bytes, so
// the FP32 form's (hi, lo) pairs, which need not be normalised, come back as
// they were and a restored case continues bit for bit.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/ibtfo.h"
#include "internal.h"

namespace ibtfo {

// density, x-vel, y-vel, pressure of the interior cells (row-major n_y x n_x);
// with `now_t` set, thread 0 also copies the loop time there
__global__ void vtk_fields_kernel(GridDesc g, const double *__restrict__ b0, const double *__restrict__ b1,
                                  const DevState *__restrict__ st, const uint8_t *__restrict__ type, float *out,
                                  double *now_t)
{
    const long long n = (long long)g.n_x * g.n_y;
    long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (now_t && c == 0)
        *now_t = st->now_t;
    if (c >= n)
        return;
    const double *buf = st->cur ? b1 : b0;
    const int j = (int)(c / g.n_x) + g.ng, i = (int)(c - (long long)(j - g.ng) * g.n_x) + g.ng;
    const long long o = (long long)j * g.pitch + i;
    float f[4] = {-1.0f, -100.0f, -100.0f, -100.0f};
    if (type[o] == CELL_FLUID || type[o] == CELL_CUT) // WriteData.cpp: cell type < 0.5 (and cut cells)
    {
        const double rho = state_ld(buf, 0, o, g);
        const double u = state_ld(buf, 1, o, g) / rho, v = state_ld(buf, 2, o, g) / rho;
        const double p = (g.gamma - 1) * (state_ld(buf, 3, o, g) - 0.5 * rho * (u * u + v * v));
        f[0] = (float)(rho > 1e-6 ? rho : 1e-6);
        f[1] = (float)u;
        f[2] = (float)v;
        f[3] = (float)p;
    }
    for (int k = 0; k < 4; k++)
        out[k * n + c] = f[k];
}

void launch_vtk_fields(const GridDesc &g, const double *b0, const double *b1, const DevState *st,
                       const uint8_t *type, float *out, double *now_t, cudaStream_t s)
{
    const long long n = (long long)g.n_x * g.n_y;
    vtk_fields_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(g, b0, b1, st, type, out, now_t);
    count_launch();
}

// VTK legacy binary data is big-endian
static void put_be_floats(FILE *f, const float *v, long long n)
{
    std::vector<uint32_t> tmp(65536);
    for (long long s = 0; s < n; s += (long long)tmp.size())
    {
        const long long m = std::min<long long>((long long)tmp.size(), n - s);
        for (long long k = 0; k < m; k++)
        {
            uint32_t x;
            std::memcpy(&x, v + s + k, 4);
            tmp[k] = (x >> 24) | ((x >> 8) & 0xFF00u) | ((x << 8) & 0xFF0000u) | (x << 24);
        }
        fwrite(tmp.data(), 4, (size_t)m, f);
    }
}

// 0, or -1 when the file cannot be written
int write_vtk_file(const char *path, const GridDesc &g, double lo_x, double lo_y, double Psy_L, double Psy_H,
                   double now_t, const float *fields, int binary)
{
    FILE *f = fopen(path, binary ? "wb" : "w");
    if (!f)
        return -1;
    const long long n = (long long)g.n_x * g.n_y;
    const double dx = Psy_L / g.n_x, dy = Psy_H / g.n_y;
    fprintf(f, "# vtk DataFile Version 2.0 \n");
    fprintf(f, "Volume example \n");
    fprintf(f, binary ? "BINARY \n" : "ASCII \n");
    fprintf(f, "DATASET STRUCTURED_POINTS \n");
    fprintf(f, "DIMENSIONS %d %d %d  \n", g.n_x, g.n_y, 1);
    fprintf(f, "ASPECT_RATIO 1 1 1 \n");
    fprintf(f, "ORIGIN %f %f %f \n", lo_x + dx / 2, lo_y + dy / 2, 0.0);
    fprintf(f, "SPACING %f %f %f \n", dx, dy, dy);
    fprintf(f, "FIELD FieldData 1  \n");
    fprintf(f, "TIME 1 1 double  \n");
    if (binary)
    {
        uint64_t x;
        std::memcpy(&x, &now_t, 8);
        uint64_t y = 0;
        for (int b = 0; b < 8; b++)
            y |= ((x >> (8 * b)) & 0xFFull) << (8 * (7 - b));
        fwrite(&y, 8, 1, f);
        fprintf(f, "\n");
    }
    else
        fprintf(f, "%f  \n", now_t);
    fprintf(f, "POINT_DATA  %lld\n", n);
    const char *names[4] = {"density", "x-vel", "y-vel", "pressure"};
    for (int k = 0; k < 4; k++)
    {
        fprintf(f, "SCALARS %s float  \n", names[k]);
        fprintf(f, "LOOKUP_TABLE default  \n");
        const float *v = fields + k * n;
        if (binary)
        {
            put_be_floats(f, v, n);
            fprintf(f, "\n");
        }
        else
            for (long long c = 0; c < n; c++)
                fprintf(f, "%f  \n", (double)v[c]);
    }
    const int ok = ferror(f) == 0;
    return (fclose(f) == 0 && ok) ? 0 : -1;
}

// Asynchronous VTK output.  submit() derives the four float fields into a
// device snapshot on the case's stream (one kernel, in order with the steps),
// then a copy stream moves the snapshot to pinned host memory while the case
// keeps stepping, and a host thread writes the file.  One write is in flight
// at a time: the next submit() or wait() joins it first, which also keeps the
// snapshot from being overwritten while it is copied.
struct VtkWriter
{
    int device = 0;
    size_t n = 0;          // interior cells
    float *dev = nullptr;  // 4*n floats, then the loop time
    float *host = nullptr; // pinned copy of dev
    cudaStream_t copy = nullptr;
    cudaEvent_t ready = nullptr, copied = nullptr;
    std::thread worker;
    int status = 0; // 0, or -1: the last finished write failed
    std::string failed;
};

static size_t snapshot_bytes(size_t n) { return ((sizeof(float) * 4 * n + 7) & ~(size_t)7) + sizeof(double); }

VtkWriter *vtk_writer_create(int device, const GridDesc &g, cudaStream_t s)
{
    VtkWriter *w = new VtkWriter;
    w->device = device;
    w->n = (size_t)g.n_x * g.n_y;
    const size_t bytes = snapshot_bytes(w->n);
    if (cudaMallocAsync(&w->dev, bytes, s) != cudaSuccess || cudaMallocHost(&w->host, bytes) != cudaSuccess ||
        cudaStreamCreateWithFlags(&w->copy, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&w->ready, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&w->copied, cudaEventDisableTiming) != cudaSuccess)
    {
        vtk_writer_destroy(w, s);
        return nullptr;
    }
    return w;
}

// joins the write in flight; 0, or -1 with `why` when a write failed since
// the last call
int vtk_writer_wait(VtkWriter *w, std::string *why)
{
    if (w->worker.joinable())
        w->worker.join();
    const int rc = w->status;
    if (rc && why)
        *why = w->failed;
    w->status = 0;
    return rc;
}

int vtk_writer_submit(VtkWriter *w, const GridDesc &g, const double *b0, const double *b1, const DevState *st,
                      const uint8_t *type, cudaStream_t s, const char *path, int binary, double lo_x, double lo_y,
                      double Psy_L, double Psy_H, std::string *why)
{
    const int prev = vtk_writer_wait(w, why);
    const size_t bytes = snapshot_bytes(w->n);
    double *t_dev = (double *)((char *)w->dev + bytes - sizeof(double));
    launch_vtk_fields(g, b0, b1, st, type, w->dev, t_dev, s);
    if (cudaGetLastError() != cudaSuccess || cudaEventRecord(w->ready, s) != cudaSuccess ||
        cudaStreamWaitEvent(w->copy, w->ready, 0) != cudaSuccess ||
        cudaMemcpyAsync(w->host, w->dev, bytes, cudaMemcpyDeviceToHost, w->copy) != cudaSuccess ||
        cudaEventRecord(w->copied, w->copy) != cudaSuccess)
    {
        if (why)
            *why = "queueing the VTK snapshot failed";
        return -1;
    }
    const std::string file(path);
    const GridDesc gd = g;
    w->worker = std::thread([w, file, gd, binary, lo_x, lo_y, Psy_L, Psy_H, bytes]() {
        cudaSetDevice(w->device);
        if (cudaEventSynchronize(w->copied) != cudaSuccess)
        {
            w->status = -1;
            w->failed = "copying the VTK snapshot failed";
            return;
        }
        double now_t;
        std::memcpy(&now_t, (const char *)w->host + bytes - sizeof(double), sizeof(double));
        if (write_vtk_file(file.c_str(), gd, lo_x, lo_y, Psy_L, Psy_H, now_t, w->host, binary))
        {
            w->status = -1;
            w->failed = "cannot write " + file;
        }
    });
    return prev;
}

void vtk_writer_destroy(VtkWriter *w, cudaStream_t s)
{
    if (!w)
        return;
    vtk_writer_wait(w, nullptr);
    if (w->copy)
    {
        cudaStreamSynchronize(w->copy);
        cudaStreamDestroy(w->copy);
    }
    if (w->ready)
        cudaEventDestroy(w->ready);
    if (w->copied)
        cudaEventDestroy(w->copied);
    if (w->host)
        cudaFreeHost(w->host);
    if (w->dev)
        cudaFreeAsync(w->dev, s);
    delete w;
}

} // namespace ibtfo
