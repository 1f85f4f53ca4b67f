// GPU-resident MD steps: nblib's leap-frog integrator and a step loop that keeps
// coordinates, velocities and forces on the device between the cluster-pair
// kernel, PME and the update.
//
// nblib::LeapFrog (api/nblib/integrator.cpp:54-77): per atom and dimension
//   v += f * dt * (1/m);  x += v * dt;   then put_atoms_in_box (pbcutil/pbc.cpp:1389-1447,
//   rectangular branch: while (x < 0) x += L; while (x >= L) x -= L).
// The kinetic energy is reported as the mean of the half-step values before and after
// the update, 0.5 (KE(t - dt/2) + KE(t + dt/2)) (the leap-frog average GROMACS uses,
// md_support.cpp compute_globals with bEkinAveVel off), summed in FP64.
//
// The step loop (nbx_md_run_device) follows do_force + update of a GPU-resident
// mdrun step (mdlib/sim_util.cpp:941-1414, 1687): nonbonded forces (search every
// nstlist steps, rolling prune), PME forces added to the same buffer, leap-frog update,
// energies every nstcalcenergy steps.  Like mdrun it puts atoms in the box only at
// search steps (the update right before one), not every step as nblib's LeapFrog does.
#include "../../include/nbnxm_gb300.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

namespace
{

constexpr int kLfThreads   = 256;
constexpr int kLfBlocksPerSm = 4;  // grid-stride; one completion-counter atomic per block
constexpr int kWrapSteps   = 4;    // box shifts applied one at a time before the floor fallback

// put_atoms_in_box for one coordinate: the reference's while loops for up to kWrapSteps
// box lengths (the same float additions), then a floor-based shift, so that a wild
// coordinate cannot keep a thread looping.
__device__ __forceinline__ float put_in_box(float x, float L)
{
    for (int k = 0; k < kWrapSteps && x < 0.0f; k++)
    {
        x = __fadd_rn(x, L);
    }
    for (int k = 0; k < kWrapSteps && x >= L; k++)
    {
        x = __fadd_rn(x, -L);
    }
    if (x < 0.0f || x >= L)
    {
        x = x - L * floorf(x / L);
        if (x < 0.0f)
        {
            x += L;
        }
        if (x >= L)
        {
            x = 0.0f;
        }
    }
    return x;
}

__global__ void __launch_bounds__(kLfThreads) k_leapfrog(int n, float dt, const float* __restrict__ inv_mass,
                                                         float* __restrict__ x, float* __restrict__ v,
                                                         const float* __restrict__ f, float3 box, int wrap,
                                                         double* partials, unsigned* done, double* ekin_out)
{
    double ke2 = 0.0;  // sum of m v^2 over the old and the new half-step velocities
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < n; a += gridDim.x * blockDim.x)
    {
        const float im    = inv_mass[a];
        const float L[3]  = { box.x, box.y, box.z };
        float       vo2   = 0.0f, vn2 = 0.0f;
        for (int d = 0; d < 3; d++)
        {
            const float vo = v[3 * a + d];
            const float vn = __fadd_rn(vo, __fmul_rn(__fmul_rn(f[3 * a + d], dt), im));
            const float xn = __fadd_rn(x[3 * a + d], __fmul_rn(vn, dt));
            v[3 * a + d]   = vn;
            x[3 * a + d]   = wrap ? put_in_box(xn, L[d]) : xn;
            vo2            = fmaf(vo, vo, vo2);
            vn2            = fmaf(vn, vn, vn2);
        }
        if (ekin_out && im > 0.0f)
        {
            ke2 += ((double)vo2 + (double)vn2) / (double)im;
        }
    }
    if (!ekin_out)
    {
        return;
    }
    __shared__ double red[kLfThreads / 32];
    __shared__ bool   last;
    const int         lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1)
    {
        ke2 += __shfl_xor_sync(0xffffffffu, ke2, o);
    }
    if (lane == 0)
    {
        red[warp] = ke2;
    }
    __syncthreads();
    if (threadIdx.x == 0)
    {
        double s = 0.0;
        for (int w = 0; w < kLfThreads / 32; w++)
        {
            s += red[w];
        }
        partials[blockIdx.x] = s;
        __threadfence();
        last = atomicAdd(done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last)
    {
        return;
    }
    __threadfence();
    double s = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
    {
        s += __ldcg(&partials[b]);
    }
    for (int o = 16; o > 0; o >>= 1)
    {
        s += __shfl_xor_sync(0xffffffffu, s, o);
    }
    __syncthreads();
    if (lane == 0)
    {
        red[warp] = s;
    }
    __syncthreads();
    if (threadIdx.x == 0)
    {
        double t = 0.0;
        for (int w = 0; w < kLfThreads / 32; w++)
        {
            t += red[w];
        }
        ekin_out[0] = 0.25 * t;  // 0.5 * (0.5 sum m vo^2 + 0.5 sum m vn^2)
        *done       = 0u;
    }
}

thread_local std::string g_md_error;

} // namespace

struct nbx_leapfrog
{
    int          device     = 0;
    int          n          = 0;
    int          num_sms    = 1;
    cudaStream_t stream     = nullptr;
    bool         own_stream = false;
    float        box[3]     = { 0, 0, 0 };
    float*       inv_mass   = nullptr;  // [N]
    double*      partials   = nullptr;  // [blocks]
    unsigned*    done       = nullptr;
    float*       d_x        = nullptr;  // host-array path staging
    float*       d_v        = nullptr;
    float*       d_f        = nullptr;
    std::string  err;
};

namespace
{

int md_error(nbx_leapfrog* p, int code, const std::string& msg)
{
    (p ? p->err : g_md_error) = msg;
    return code;
}

int lf_blocks(const nbx_leapfrog* p)
{
    return std::max(1, std::min((p->n + kLfThreads - 1) / kLfThreads, kLfBlocksPerSm * p->num_sms));
}

int launch_leapfrog(nbx_leapfrog* p, float dt, float* d_x, float* d_v, const float* d_f, double* d_ekin, int wrap)
{
    if (p->n == 0)
    {
        return NBX_OK;
    }
    cudaSetDevice(p->device);
    k_leapfrog<<<lf_blocks(p), kLfThreads, 0, p->stream>>>(p->n, dt, p->inv_mass, d_x, d_v, d_f,
                                                           make_float3(p->box[0], p->box[1], p->box[2]), wrap,
                                                           p->partials, p->done, d_ekin);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? NBX_OK : md_error(p, NBX_ERR_CUDA, cudaGetErrorString(e));
}

} // namespace

namespace
{
int run_steps(nbx_handle* h, nbx_pme* pme, nbx_leapfrog* lf, long long first_step, int num_steps, float dt,
              float* d_x, float* d_v, float* d_f, const float* d_q, int nstcalcenergy, double* d_energies,
              int nstlist, int natoms, void* s);
} // namespace

extern "C" {

const char* nbx_leapfrog_last_error(const nbx_leapfrog* p)
{
    return p ? p->err.c_str() : g_md_error.c_str();
}

int nbx_leapfrog_create(int num_atoms, const float* inv_mass, const float* box, int device, nbx_leapfrog** out)
{
    if (!out || num_atoms < 0 || (num_atoms > 0 && !inv_mass) || !box)
    {
        return md_error(nullptr, NBX_ERR_INVALID_INPUT, "null argument or negative atom count");
    }
    *out = nullptr;
    for (int k = 0; k < 3; k++)
    {
        if (!(box[k] > 0.0f))
        {
            return md_error(nullptr, NBX_ERR_INVALID_INPUT, "box edges must be positive");
        }
    }
    for (int a = 0; a < num_atoms; a++)
    {
        if (!(inv_mass[a] >= 0.0f) || std::isinf(inv_mass[a]))
        {
            return md_error(nullptr, NBX_ERR_INVALID_INPUT, "inverse masses must be finite and >= 0");
        }
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    {
        cudaGetLastError();
        return md_error(nullptr, NBX_ERR_NO_DEVICE, "no CUDA device");
    }
    if (device < 0 || device >= ndev)
    {
        return md_error(nullptr, NBX_ERR_INVALID_INPUT, "device index out of range");
    }
    cudaSetDevice(device);
    nbx_leapfrog* p = new nbx_leapfrog();
    p->device       = device;
    p->n            = num_atoms;
    for (int k = 0; k < 3; k++)
    {
        p->box[k] = box[k];
    }
    cudaError_t e = cudaDeviceGetAttribute(&p->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking);
    p->own_stream = e == cudaSuccess;
    const size_t bytes = sizeof(float) * std::max(1, num_atoms);
    if (e == cudaSuccess) e = cudaMalloc(&p->inv_mass, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&p->partials, sizeof(double) * kLfBlocksPerSm * p->num_sms);
    if (e == cudaSuccess) e = cudaMalloc(&p->done, sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMemset(p->done, 0, sizeof(unsigned));
    if (e == cudaSuccess && num_atoms > 0) e = cudaMemcpy(p->inv_mass, inv_mass, bytes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess)
    {
        const std::string msg = cudaGetErrorString(e);
        nbx_leapfrog_destroy(p);
        return md_error(nullptr, NBX_ERR_OUT_OF_MEMORY, "leap-frog allocation: " + msg);
    }
    *out = p;
    return NBX_OK;
}

int nbx_leapfrog_destroy(nbx_leapfrog* p)
{
    if (!p)
    {
        return NBX_OK;
    }
    cudaSetDevice(p->device);
    if (p->stream)
    {
        cudaStreamSynchronize(p->stream);
    }
    cudaFree(p->inv_mass);
    cudaFree(p->partials);
    cudaFree(p->done);
    cudaFree(p->d_x);
    cudaFree(p->d_v);
    cudaFree(p->d_f);
    if (p->own_stream)
    {
        cudaStreamDestroy(p->stream);
    }
    delete p;
    return NBX_OK;
}

int nbx_leapfrog_set_stream(nbx_leapfrog* p, void* s)
{
    if (!p)
    {
        return md_error(nullptr, NBX_ERR_INVALID_INPUT, "null handle");
    }
    if (static_cast<cudaStream_t>(s) == p->stream)
    {
        return NBX_OK;
    }
    cudaSetDevice(p->device);
    cudaStreamSynchronize(p->stream);
    if (p->own_stream)
    {
        cudaStreamDestroy(p->stream);
    }
    p->stream     = static_cast<cudaStream_t>(s);
    p->own_stream = false;
    return NBX_OK;
}

int nbx_leapfrog_integrate_device(nbx_leapfrog* p, float dt, float* d_x, float* d_v, const float* d_f,
                                  double* d_ekin)
{
    if (!p || (p->n > 0 && (!d_x || !d_v || !d_f)) || !std::isfinite(dt))
    {
        return md_error(p, NBX_ERR_INVALID_INPUT, "null argument or non-finite time step");
    }
    return launch_leapfrog(p, dt, d_x, d_v, d_f, d_ekin, 1);
}

int nbx_leapfrog_integrate(nbx_leapfrog* p, float dt, float* x, float* v, const float* f)
{
    if (!p || (p->n > 0 && (!x || !v || !f)))
    {
        return md_error(p, NBX_ERR_INVALID_INPUT, "null argument");
    }
    if (p->n == 0)
    {
        return NBX_OK;
    }
    cudaSetDevice(p->device);
    const size_t bytes = sizeof(float) * 3 * p->n;
    cudaError_t  e     = cudaSuccess;
    if (!p->d_x)
    {
        e = cudaMalloc(&p->d_x, bytes);
        if (e == cudaSuccess) e = cudaMalloc(&p->d_v, bytes);
        if (e == cudaSuccess) e = cudaMalloc(&p->d_f, bytes);
        if (e != cudaSuccess)
        {
            return md_error(p, NBX_ERR_OUT_OF_MEMORY, cudaGetErrorString(e));
        }
    }
    e = cudaMemcpyAsync(p->d_x, x, bytes, cudaMemcpyHostToDevice, p->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(p->d_v, v, bytes, cudaMemcpyHostToDevice, p->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(p->d_f, f, bytes, cudaMemcpyHostToDevice, p->stream);
    if (e != cudaSuccess)
    {
        return md_error(p, NBX_ERR_CUDA, cudaGetErrorString(e));
    }
    const int rc = nbx_leapfrog_integrate_device(p, dt, p->d_x, p->d_v, p->d_f, nullptr);
    if (rc != NBX_OK)
    {
        return rc;
    }
    e = cudaMemcpyAsync(x, p->d_x, bytes, cudaMemcpyDeviceToHost, p->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(v, p->d_v, bytes, cudaMemcpyDeviceToHost, p->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(p->stream);
    return e == cudaSuccess ? NBX_OK : md_error(p, NBX_ERR_CUDA, cudaGetErrorString(e));
}

int nbx_md_run_device(nbx_handle* h, nbx_pme* pme, nbx_leapfrog* lf, long long first_step, int num_steps, float dt,
                      float* d_x, float* d_v, float* d_f, const float* d_q, int nstcalcenergy, double* d_energies)
{
    if (!h || !lf || num_steps < 0 || !d_x || !d_v || !d_f || (pme && !d_q) || !std::isfinite(dt)
        || (d_energies && nstcalcenergy < 1))
    {
        return md_error(lf, NBX_ERR_INVALID_INPUT, "null argument, negative step count or bad nstcalcenergy");
    }
    // one stream for the whole step: the nonbonded handle's
    void* s  = nbx_get_stream(h);
    int   rc = nbx_leapfrog_set_stream(lf, s);
    if (rc == NBX_OK && pme)
    {
        rc = nbx_pme_set_stream(pme, s);
    }
    if (rc != NBX_OK)
    {
        return rc;
    }
    int natoms = 0;
    {
        int sizes[8];
        if ((rc = nbx_get_sizes(h, sizes)) != NBX_OK)
        {
            return rc;
        }
        natoms = sizes[0];
    }
    if (natoms != lf->n)
    {
        return md_error(lf, NBX_ERR_INVALID_INPUT, "the leap-frog and nonbonded handles differ in atom count");
    }
    nbx_options opts;
    if ((rc = nbx_get_options(h, &opts)) != NBX_OK)
    {
        return rc;
    }
    const int nstlist = std::max(1, opts.nstlist);
    // each step starts a fresh force buffer: the nonbonded forces overwrite it
    int accumulate = 0;
    nbx_get_force_accumulate(h, &accumulate);
    nbx_set_force_accumulate(h, 0);
    rc = run_steps(h, pme, lf, first_step, num_steps, dt, d_x, d_v, d_f, d_q, nstcalcenergy, d_energies, nstlist,
                   natoms, s);
    nbx_set_force_accumulate(h, accumulate);
    return rc;
}

} // extern "C"

namespace
{

int run_steps(nbx_handle* h, nbx_pme* pme, nbx_leapfrog* lf, long long first_step, int num_steps, float dt,
              float* d_x, float* d_v, float* d_f, const float* d_q, int nstcalcenergy, double* d_energies,
              int nstlist, int natoms, void* s)
{
    int rc = NBX_OK;
    for (int k = 0; k < num_steps; k++)
    {
        const long long step   = first_step + k;
        const bool      energy = d_energies && (step - first_step) % nstcalcenergy == 0;
        double*         row    = energy ? d_energies + 4 * ((step - first_step) / nstcalcenergy) : nullptr;
        // row: {E_LJ, E_Coulomb real space (incl. self and exclusion corrections), E_Coulomb reciprocal, E_kin}
        if ((rc = nbx_md_step_device(h, step, d_x, d_f, row, nullptr)) != NBX_OK)
        {
            return rc;
        }
        if (pme && (rc = nbx_pme_compute_device(pme, natoms, d_x, d_q, d_f, row ? row + 2 : nullptr, nullptr)) != NBX_OK)
        {
            return rc;
        }
        if (row && !pme && cudaMemsetAsync(row + 2, 0, sizeof(double), static_cast<cudaStream_t>(s)) != cudaSuccess)
        {
            return md_error(lf, NBX_ERR_CUDA, "energy row");
        }
        // put_atoms_in_box only right before a search step: the nonbonded handle keeps each
        // atom's box shift from the last search (like mdrun, which wraps at search steps)
        const int wrap = (step + 1) % nstlist == 0 ? 1 : 0;
        if ((rc = launch_leapfrog(lf, dt, d_x, d_v, d_f, row ? row + 3 : nullptr, wrap)) != NBX_OK)
        {
            return rc;
        }
    }
    return NBX_OK;
}

} // namespace
