// Instantiations and launcher of the mixed-precision work-list contraction (k_mixed.cuh).
#include "k_mixed.cuh"

namespace mwgpu {

namespace {
template <int K>
void launch_k(const DevMRA &m, const DevOper &op, const DevTree &f, DevTree g, const int *work, const int4 *chunks, int n_chunks,
              const WorkItem *items, double *partial, int *err, cudaStream_t s) {
    size_t smem = sizeof(float) * mixed::Shape<K>::SMEM_FLOATS;
    auto kern = mixed::k_contract_items<K>;
    if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    kern<<<n_chunks, 256, smem, s>>>(m, op, f, g, work, chunks, items, partial, err);
}
}  // namespace

bool mixed_supported(int K) { return K >= 2 && K <= 12; }

void launch_items(const DevMRA &m, const DevOper &op, const DevTree &f, DevTree g, const int *work, const int4 *chunks, int n_chunks,
                  const WorkItem *items, double *partial, int *err, cudaStream_t s);

void launch_contract_items(const DevMRA &m, const DevOper &op, const DevTree &f, DevTree g, const int *work, int n_work, const int4 *chunks,
                           int n_chunks, const int *chunk_begin, const WorkItem *items, double *partial, int *err, cudaStream_t s) {
    if (n_work <= 0) return;
    launch_items(m, op, f, g, work, chunks, n_chunks, items, partial, err, s);
    mixed::k_reduce_chunks<<<n_work, 256, 0, s>>>(g, work, chunk_begin, partial, 8 * m.kp1_d);
}

void launch_items(const DevMRA &m, const DevOper &op, const DevTree &f, DevTree g, const int *work, const int4 *chunks, int n_chunks,
                  const WorkItem *items, double *partial, int *err, cudaStream_t s) {
    if (n_chunks <= 0) return;
    switch (m.K) {
        case 2: launch_k<2>(m, op, f, g, work, chunks, n_chunks, items, partial, err, s); break;
        case 3: launch_k<3>(m, op, f, g, work, chunks, n_chunks, items, partial, err, s); break;
        case 4: launch_k<4>(m, op, f, g, work, chunks, n_chunks, items, partial, err, s); break;
        case 5: launch_k<5>(m, op, f, g, work, chunks, n_chunks, items, partial, err, s); break;
        case 6: launch_k<6>(m, op, f, g, work, chunks, n_chunks, items, partial, err, s); break;
        case 7: launch_k<7>(m, op, f, g, work, chunks, n_chunks, items, partial, err, s); break;
        case 8: launch_k<8>(m, op, f, g, work, chunks, n_chunks, items, partial, err, s); break;
        case 9: launch_k<9>(m, op, f, g, work, chunks, n_chunks, items, partial, err, s); break;
        case 10: launch_k<10>(m, op, f, g, work, chunks, n_chunks, items, partial, err, s); break;
        case 11: launch_k<11>(m, op, f, g, work, chunks, n_chunks, items, partial, err, s); break;
        case 12: launch_k<12>(m, op, f, g, work, chunks, n_chunks, items, partial, err, s); break;
        default: break;
    }
}

}  // namespace mwgpu
