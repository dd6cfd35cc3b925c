// Golden vectors of the GPU's stochastic-rounding FP16 conversion
// (cvt.rs.f16x2.f32), which the FP16-SR storage of the LBM kernels uses and
// the oracle restates (oracle/lbm_oracle.hpp, f32_to_f16_sr). Test
// infrastructure: run on a GB300 from the repository root,
//   nvcc -gencode arch=compute_103a,code=sm_103a -o /tmp/f16rs tests/golden/make_f16_rs_golden.cu && /tmp/f16rs
// which writes tests/golden/f16_rs_golden.bin: int32 n, then n floats a
// (high result), n floats b (low result), n uint32 random words, n uint32
// results. Cases: a scan of one-bit random words against remainders
// 8192 - 2^j at 1 + D 2^-23 (which bits feed which half, and their weight),
// then seeded random values of both signs over normal FP16 magnitudes, the
// FP16 subnormal range and 2^14 .. 2^18 (rounding past the largest finite
// value).
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

__global__ void convert(const float* a, const float* b, const uint32_t* r, uint32_t* o, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t w;
    asm("cvt.rs.f16x2.f32 %0, %1, %2, %3;" : "=r"(w) : "f"(a[i]), "f"(b[i]), "r"(r[i]));
    o[i] = w;
}

static uint32_t next(uint64_t& s)
{
    s = s * 6364136223846793005ull + 1442695040888963407ull;
    return uint32_t(s >> 32);
}

static float from_bits(uint32_t u)
{
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

int main()
{
    std::vector<float>    A, B;
    std::vector<uint32_t> R;
    for (int j = 0; j <= 13; j++) {
        const uint32_t D = j == 13 ? 0u : 8192u - (1u << j);
        for (int k = 0; k < 32; k++) {
            A.push_back(from_bits(0x3f800000u + D));
            B.push_back(from_bits(0x3f800000u + D));
            R.push_back(1u << k);
        }
    }
    uint64_t s = 20261204;
    while (A.size() < 16384) {
        const bool     sub = A.size() % 4 == 0;  // a quarter in the FP16 subnormal range
        const bool     big = A.size() % 16 == 1; // some at 2^14 .. 2^18 (overflow past 65504)
        const uint32_t ea = sub ? 0x30000000u + next(s) % 0x08800000u
                                : (big ? 0x46800000u + next(s) % 0x02000000u : 0x38800000u + next(s) % 0x0f000000u);
        const uint32_t eb = sub ? 0x30000000u + next(s) % 0x08800000u
                                : (big ? 0x46800000u + next(s) % 0x02000000u : 0x38800000u + next(s) % 0x0f000000u);
        A.push_back(from_bits((ea & 0xff800000u) | (next(s) & 0x7fffffu) | ((next(s) & 1u) << 31)));
        B.push_back(from_bits((eb & 0xff800000u) | (next(s) & 0x7fffffu) | ((next(s) & 1u) << 31)));
        R.push_back(next(s));
    }
    const int n = int(A.size());
    float *   da, *db;
    uint32_t *dr, *dout;
    if (cudaMalloc(&da, n * 4) != cudaSuccess || cudaMalloc(&db, n * 4) != cudaSuccess || cudaMalloc(&dr, n * 4) != cudaSuccess ||
        cudaMalloc(&dout, n * 4) != cudaSuccess)
        return 1;
    cudaMemcpy(da, A.data(), n * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(db, B.data(), n * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(dr, R.data(), n * 4, cudaMemcpyHostToDevice);
    convert<<<(n + 255) / 256, 256>>>(da, db, dr, dout, n);
    if (cudaDeviceSynchronize() != cudaSuccess) return 1;
    std::vector<uint32_t> O(n);
    cudaMemcpy(O.data(), dout, n * 4, cudaMemcpyDeviceToHost);
    FILE* f = std::fopen("tests/golden/f16_rs_golden.bin", "wb");
    if (!f) return 1;
    std::fwrite(&n, 4, 1, f);
    std::fwrite(A.data(), 4, n, f);
    std::fwrite(B.data(), 4, n, f);
    std::fwrite(R.data(), 4, n, f);
    std::fwrite(O.data(), 4, n, f);
    std::fclose(f);
    std::printf("wrote tests/golden/f16_rs_golden.bin (%d cases)\n", n);
    return 0;
}
