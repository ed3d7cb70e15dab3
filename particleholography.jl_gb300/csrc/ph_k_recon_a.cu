// Reconstruction pass A: per-slice transfer + inverse FFT along ky, transposed store.
#include "ph_launch.cuh"

namespace ph {

int recon_a_rows(int n) {
    switch (n) {
#define PH_ROWS_A(N) case N: return Shape<N, ReconA::EPT, ReconA::TT>::ROWS;
        PH_FOR_EACH_N(PH_ROWS_A)
#undef PH_ROWS_A
    }
    return 1;
}

bool recon_a_chain(int n, bool tstore) {
    if (tstore) {
        switch (n) {
#define PH_CHAIN_AT(N) case N: return ReconATStore::form<N, true>() == ReconATStore::FORM_CHAIN;
            PH_CHAIN_AT(256) PH_CHAIN_AT(512) PH_CHAIN_AT(1024) PH_CHAIN_AT(2048) PH_CHAIN_AT(4096)
#undef PH_CHAIN_AT
        }
    }
    switch (n) {
#define PH_CHAIN_A(N) case N: return ReconA::form<N, true>() == ReconA::FORM_CHAIN;
        PH_FOR_EACH_N(PH_CHAIN_A)
#undef PH_CHAIN_A
    }
    return false;
}

cudaError_t launch_recon_a(int n, const ReconA &b, int nbatch, cudaStream_t s) {
    return launch_len<true>(n, b, b.nx, (nbatch + b.group - 1) / b.group, s);
}

// The tensor-map form: CTAs of 8192 / n rows at 256 .. 2048, clusters of two
// 2-row CTAs at 4096.
bool recon_a_tstore(int n) { return n == 256 || n == 512 || n == 1024 || n == 2048 || n == 4096; }

// kx per box of that form: the rows of a CTA, or of a cluster.
int recon_a_tstore_box(int n) {
    switch (n) {
#define PH_BOX_A(N) case N: return Shape<N, ReconATStore::EPT, ReconATStore::TT>::ROWS * ReconATStore::cluster<N>();
        PH_BOX_A(256) PH_BOX_A(512) PH_BOX_A(1024) PH_BOX_A(2048) PH_BOX_A(4096)
#undef PH_BOX_A
    }
    return 0;
}

cudaError_t launch_recon_a_tstore(int n, const ReconATStore &b, const CUtensorMap &tm, int nbatch, cudaStream_t s) {
    const int gy = (nbatch + b.group - 1) / b.group;
    switch (n) {
        case 256: return launch_one_tm<256, true>(b, tm, b.nx, gy, s);
        case 512: return launch_one_tm<512, true>(b, tm, b.nx, gy, s);
        case 1024: return launch_one_tm<1024, true>(b, tm, b.nx, gy, s);
        case 2048: return launch_one_tm<2048, true>(b, tm, b.nx, gy, s);
        case 4096: return launch_one_tm<4096, true>(b, tm, b.nx, gy, s);
    }
    return cudaErrorInvalidValue;
}

}  // namespace ph
