// Prints the permutation thrust::shuffle(first, last, thrust::default_random_engine()) applies to
// [0, m) for each m given on the command line, one line per m: "m p0 p1 ...". Built against the CCCL
// headers of the CUDA toolkit with the CPP device system (the generic shuffle algorithm is shared by the
// host and CUDA backends), it pins the oracle's restatement of the shuffle used at the reference's
// cusimp_free.cu:937-941.
#include <thrust/device_vector.h>
#include <thrust/random.h>
#include <thrust/sequence.h>
#include <thrust/shuffle.h>
#include <cstdio>
#include <cstdlib>

int main(int argc, char** argv) {
    for (int a = 1; a < argc; ++a) {
        long m = std::atol(argv[a]);
        thrust::device_vector<int> v(m);
        thrust::sequence(v.begin(), v.end());
        thrust::default_random_engine rng;
        thrust::shuffle(v.begin(), v.end(), rng);
        std::printf("%ld", m);
        for (long i = 0; i < m; ++i) std::printf(" %d", (int)v[i]);
        std::printf("\n");
    }
    return 0;
}
