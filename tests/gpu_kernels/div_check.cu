// Exhaustive checks of the AMAZE weight arithmetic against CUDA's correctly rounded operations:
//   dev::rcp_small_int(n) against __frcp_rn(n) for every n in [1, 3 * 65535 + 1];
//   dev::weight_quotients against __fdiv_rn over every pair of weights a = 1/(1+gH),
//   b = 1/(1+gV), gH, gV in [0, 3 (2^bd - 1)] for the bit depth given (default 12).
// Built and run by tests/test_gpu_division.py; prints the mismatch counts and exits non-zero on
// any mismatch.
#include <cstdio>
#include <cstdlib>

#include "../../im-operator_gb300/csrc/isp_device.cuh"

__global__ void check_rcp(int nmax, unsigned long long* bad) {
    for (int n = 1 + blockIdx.x * blockDim.x + threadIdx.x; n <= nmax; n += gridDim.x * blockDim.x)
        if (imop::dev::rcp_small_int(n) != __frcp_rn((float)n)) atomicAdd(bad, 1ull);
}

__global__ void check_pairs(long long n, float neg_zero, unsigned long long* bad, long long* first) {
    const float2 z2 = make_float2(neg_zero, neg_zero);
    const long long total = n * n;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int gh = (int)(i / n), gv = (int)(i - (i / n) * n);
        const float a = imop::dev::rcp_small_int(1 + gh), b = imop::dev::rcp_small_int(1 + gv);
        const float s = __fadd_rn(a, b);
        const float2 w = imop::dev::weight_quotients(a, b, z2);
        if (w.x != __fdiv_rn(a, s) || w.y != __fdiv_rn(b, s)) {
            atomicAdd(bad, 1ull);
            atomicMin(reinterpret_cast<unsigned long long*>(first), (unsigned long long)i);
        }
    }
}

int main(int argc, char** argv) {
    const int bd = argc > 1 ? atoi(argv[1]) : 12;
    const long long n = 3LL * ((1LL << bd) - 1) + 1;
    unsigned long long* bad = nullptr;
    unsigned long long* bad_rcp = nullptr;
    long long* first = nullptr;
    if (cudaMalloc(&bad, sizeof(*bad)) || cudaMalloc(&bad_rcp, sizeof(*bad_rcp)) || cudaMalloc(&first, sizeof(*first)))
        return 2;
    const long long init_first = 0x7fffffffffffffffLL;
    cudaMemset(bad, 0, sizeof(*bad));
    cudaMemset(bad_rcp, 0, sizeof(*bad_rcp));
    cudaMemcpy(first, &init_first, sizeof(init_first), cudaMemcpyHostToDevice);
    const int nmax = 3 * 65535 + 1;
    check_rcp<<<152, 256>>>(nmax, bad_rcp);
    check_pairs<<<152 * 8, 256>>>(n, -0.0f, bad, first);
    unsigned long long nb = 0, nr = 0;
    long long f = 0;
    if (cudaMemcpy(&nb, bad, sizeof(nb), cudaMemcpyDeviceToHost) || cudaMemcpy(&nr, bad_rcp, sizeof(nr), cudaMemcpyDeviceToHost) ||
        cudaMemcpy(&f, first, sizeof(f), cudaMemcpyDeviceToHost))
        return 3;
    printf("reciprocals 1..%d: %llu mismatches\n", nmax, nr);
    printf("bit depth %d: %lld weight pairs, %llu mismatches", bd, n * n, nb);
    if (nb) printf(" (first gradH %lld gradV %lld)", f / n, f % n);
    printf("\n");
    return (nb || nr) ? 1 : 0;
}
