// Instantiations and launcher of the mixed-precision work-list contraction (k_mixed.cuh).
#include <cstdlib>

#include "k_mixed.cuh"

namespace mwgpu {

namespace {
template <int K>
void launch_k(const DevMRA &m, const DevOper &op, const DevTree *fs, const DevTree *gs, const int *work_tree, const int *work, const int4 *chunks,
              int n_chunks, const WorkItem *items, double *partial, int *err, const int *n_chunks_dev, int *counter, cudaStream_t s) {
    size_t smem = sizeof(float) * mixed::Shape<K>::SMEM_FLOATS;
    auto kern = mixed::k_contract_items<K>;
    if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    kern<<<n_chunks, mixed::Shape<K>::NT, smem, s>>>(m, op, fs, gs, work_tree, work, chunks, items, partial, err, n_chunks_dev, counter);
}

template <int K>
int resident_k() {
    size_t smem = sizeof(float) * mixed::Shape<K>::SMEM_FLOATS;
    auto kern = mixed::k_contract_items<K>;
    if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, mixed::Shape<K>::NT, smem) != cudaSuccess) return 0;
    return nb;
}
}  // namespace

// the staged blocks of K >= 11 do not fit the 227 KB of shared memory of a CTA
bool mixed_supported(int K) { return K >= 2 && K <= 10; }


void launch_contract_items(const DevMRA &m, const DevOper &op, const DevTree *fs, const DevTree *gs, const int *work_tree, const int *work,
                           int n_work, const int4 *chunks, int n_chunks, const int *chunk_begin, const WorkItem *items, double *partial, int *err,
                           int *tc_counter, cudaStream_t s) {
    if (n_work <= 0) return;
    launch_items(m, op, fs, gs, work_tree, work, chunks, n_chunks, items, partial, err, nullptr, nullptr, tc_counter, s);
    mixed::k_reduce_chunks<<<dim3(n_work, 8), mixed::kReduceThreads, 0, s>>>(gs, work_tree, work, chunk_begin, partial, 8 * m.kp1_d, nullptr);
}

void launch_reduce_chunks(const DevMRA &m, const DevTree *gs, const int *work_tree, const int *work, int n_work, const int *chunk_begin,
                          const double *partial, cudaStream_t s, const int *nw_dev, const int *pen_begin, const double *pen_partial) {
    if (n_work <= 0) return;
    mixed::k_reduce_chunks<<<dim3(n_work, 8), mixed::kReduceThreads, 0, s>>>(gs, work_tree, work, chunk_begin, partial, 8 * m.kp1_d, nw_dev,
                                                                             pen_begin, pen_partial);
}

int contract_items_resident(int K) {
    switch (K) {
        case 2: return resident_k<2>();
        case 3: return resident_k<3>();
        case 4: return resident_k<4>();
        case 5: return resident_k<5>();
        case 6: return resident_k<6>();
        case 7: return resident_k<7>();
        case 8: return resident_k<8>();
        case 9: return resident_k<9>();
        case 10: return resident_k<10>();
        default: return 0;
    }
}

void launch_items(const DevMRA &m, const DevOper &op, const DevTree *fs, const DevTree *gs, const int *work_tree, const int *work,
                  const int4 *chunks, int n_chunks, const WorkItem *items, double *partial, int *err, const int *n_chunks_dev, int *counter,
                  int *tc_counter, cudaStream_t s) {
    if (n_chunks <= 0) return;
    // order 7 with MWGPU_TC set: chunks of block-schedule items go to the
    // tcgen05 kernel (k_tc.cu), the others (screened items) to the kernel below
    // (the input trees of the level carry their TF32 operands only when they
    // were uploaded with MWGPU_TC set; the kernel reads them from fs[tree].tc32)
    const bool tc = tc_supported(m.K) && op.btc && tc_counter && std::getenv("MWGPU_TC");
    if (tc) launch_chunk_types(const_cast<int4 *>(chunks), n_chunks, n_chunks_dev, items, s);
    switch (m.K) {
        case 2: launch_k<2>(m, op, fs, gs, work_tree, work, chunks, n_chunks, items, partial, err, n_chunks_dev, counter, s); break;
        case 3: launch_k<3>(m, op, fs, gs, work_tree, work, chunks, n_chunks, items, partial, err, n_chunks_dev, counter, s); break;
        case 4: launch_k<4>(m, op, fs, gs, work_tree, work, chunks, n_chunks, items, partial, err, n_chunks_dev, counter, s); break;
        case 5: launch_k<5>(m, op, fs, gs, work_tree, work, chunks, n_chunks, items, partial, err, n_chunks_dev, counter, s); break;
        case 6: launch_k<6>(m, op, fs, gs, work_tree, work, chunks, n_chunks, items, partial, err, n_chunks_dev, counter, s); break;
        case 7: launch_k<7>(m, op, fs, gs, work_tree, work, chunks, n_chunks, items, partial, err, n_chunks_dev, counter, s); break;
        case 8: launch_k<8>(m, op, fs, gs, work_tree, work, chunks, n_chunks, items, partial, err, n_chunks_dev, counter, s); break;
        case 9: launch_k<9>(m, op, fs, gs, work_tree, work, chunks, n_chunks, items, partial, err, n_chunks_dev, counter, s); break;
        case 10: launch_k<10>(m, op, fs, gs, work_tree, work, chunks, n_chunks, items, partial, err, n_chunks_dev, counter, s); break;
        default: break;
    }
    if (tc) launch_contract_tc(m, op, fs, gs, work_tree, work, chunks, n_chunks, n_chunks_dev, items, partial, err, tc_counter, s);
}

}  // namespace mwgpu
