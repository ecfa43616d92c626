"""oracle/cuda_emu.py, the host emulation that runs the reference's CUDA
kernel strings for the parity fixtures: its two launch modes, barriers past
threads that returned, atomics, and texture fetches.  CPU only (g++)."""
import numpy as np
import pytest

from oracle import cuda_emu

# every thread reads what another thread of its block wrote before the barrier
REVERSE = r"""
__global__ void reverse(float* out, int n)
{
    __shared__ float buf[64];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    buf[threadIdx.x] = i < n ? 10.0f * i : -1.0f;
    __syncthreads();
    if (i < n) out[i] = buf[blockDim.x - 1 - threadIdx.x];
}
"""

# threads past the end return before two barriers; the rest sum a tile
EARLY = r"""
__global__ void partial_sums(const float* in, float* out, float* total, int n)
{
    __shared__ float tile[32];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    tile[threadIdx.x] = in[i];
    __syncthreads();
    if (threadIdx.x == 0) {
        float s = 0;
        for (int k = 0; k < 32 && blockIdx.x * blockDim.x + k < n; ++k) s += tile[k];
        out[blockIdx.x] = s;
    }
    __syncthreads();
    atomicAdd(total, in[i]);
}
"""

TEXTURE = r"""
texture<fp_tex_float, cudaTextureType3D, cudaReadModeElementType> tex;
__global__ void fetch(const float* xyz, float* out, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = fp_tex3D(tex, xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
}
"""


def test_barriers_order_shared_memory_both_ways():
    n = 100
    out = np.zeros(n, dtype=np.float32)
    cuda_emu.Module(REVERSE, barriers=True).get_function("reverse")(
        out, np.int32(n), block=(32, 1, 1), grid=(4, 1))
    want = np.empty(n, dtype=np.float32)
    for i in range(n):
        b, t = divmod(i, 32)
        j = b * 32 + 31 - t
        want[i] = 10.0 * j if j < n else -1.0
    np.testing.assert_array_equal(out, want)


def test_sequential_mode_runs_threads_in_order():
    # without a real barrier, a thread reads its partner's slot before the
    # partner wrote it this launch: the documented limit of sequential mode
    n = 64
    out = np.zeros(n, dtype=np.float32)
    cuda_emu.Module(REVERSE).get_function("reverse")(out, np.int32(n), block=(32, 1, 1),
                                                    grid=(2, 1))
    # the first thread of each block reads slot 31 before its writer runs
    assert out[0] != 10.0 * 31 and out[32] != 10.0 * 63


def test_returned_threads_leave_the_barrier_and_atomics_add():
    n = 70
    x = np.arange(1, n + 1, dtype=np.float32)
    out = np.zeros(3, dtype=np.float32)
    total = np.zeros(1, dtype=np.float32)
    cuda_emu.Module(EARLY, barriers=True).get_function("partial_sums")(
        x, out, total, np.int32(n), block=(32, 1, 1), grid=(3, 1))
    np.testing.assert_array_equal(out, [x[:32].sum(), x[32:64].sum(), x[64:].sum()])
    assert total[0] == x.sum()


@pytest.mark.parametrize("barriers", [False, True])
def test_texture_fetch_is_point_sampled_and_clamped(barriers):
    d, h, w = 2, 3, 4
    arr = np.arange(d * h * w, dtype=np.float32).reshape(d, h, w)
    mod = cuda_emu.Module(TEXTURE, barriers=barriers)
    mod.get_texref("tex").set_array(arr)
    pts = np.array([[0.5, 0.5, 0.5], [3.99, 2.2, 1.7], [1.0, 1.0, 0.0], [-3.0, 7.0, 9.0],
                    [2.5, 0.0, 1.2]], dtype=np.float32)
    out = np.zeros(len(pts), dtype=np.float32)
    mod.get_function("fetch")(pts, out, np.int32(len(pts)), block=(8, 1, 1), grid=(1, 1))
    ix = np.clip(np.floor(pts).astype(int), 0, [w - 1, h - 1, d - 1])
    np.testing.assert_array_equal(out, arr[ix[:, 2], ix[:, 1], ix[:, 0]])
