/*
 * CPU restatement of the reference's connected-component labeling -- TEST
 * INFRASTRUCTURE ONLY (the oracle; never linked into the product library).
 *
 * Follows ParticleHolography.jl src/ccl.jl, which is the Playne-Hawick 8-way
 * label-equivalence algorithm (after FolkeV/CUDA_CCL):
 *   find_root          ccl.jl:13-25
 *   reduction          ccl.jl:28-67   (atomicMin union; old value returned)
 *   init_labels        ccl.jl:70-98
 *   resolve_labels     ccl.jl:100-113
 *   label_reduction    ccl.jl:115-157
 *   resolve_background ccl.jl:159-172
 *   driver             ccl.jl:186-211
 * Each kernel is executed here as a sequential loop over the pixels.  The
 * algorithm's result does not depend on the order the pixels are visited in:
 * every pixel ends up labelled with the minimum linear index of its
 * 8-connected equal-valued component, plus one, and background pixels
 * (value <= 0) are set to 0.
 *
 * The buffer is viewed as a C-row-major grid of `rows` x `cols` elements: the
 * reference's `numRows = height = size(img,1)` and `numCols = width =
 * size(img,2)` over the column-major buffer, i.e. index `iy*numCols + ix`.
 */
#include <stdint.h>

static uint32_t find_root(const uint32_t *labels, uint32_t label)
{
    uint32_t next = labels[label];
    while (label != next) {
        label = next;
        next = labels[label];
    }
    return label;
}

static uint32_t atomic_min_seq(uint32_t *p, uint32_t v)
{
    uint32_t old = *p;
    if (v < old) *p = v;
    return old;
}

static uint32_t reduction(uint32_t *labels, uint32_t label1, uint32_t label2)
{
    uint32_t next1 = (label1 != label2) ? labels[label1] : 1;
    uint32_t next2 = (label1 != label2) ? labels[label2] : 1;
    while (label1 != label2 && label1 != next1) {
        label1 = next1;
        next1 = labels[label1];
    }
    while (label1 != label2 && label2 != next2) {
        label2 = next2;
        next2 = labels[label2];
    }
    while (label1 != label2) {
        if (label1 < label2) {
            uint32_t t = label1;
            label1 = label2;
            label2 = t;
        }
        uint32_t label3 = atomic_min_seq(&labels[label1], label2);
        label1 = (label1 == label3) ? label2 : label3;
    }
    return label1;
}

/* img: rows*cols float32 values; labels: rows*cols uint32 output. */
void oracle_ccl_f32(const float *img, uint32_t *labels, int64_t rows, int64_t cols)
{
    int64_t iy, ix;
    /* init_labels */
    for (iy = 0; iy < rows; ++iy) {
        for (ix = 0; ix < cols; ++ix) {
            float p = img[iy * cols + ix];
            int n_n = (iy > 0) && (p == img[(iy - 1) * cols + ix]);
            int n_w = (ix > 0) && (p == img[iy * cols + ix - 1]);
            int n_nw = (iy > 0) && (ix > 0) && (p == img[(iy - 1) * cols + ix - 1]);
            int n_ne = (iy > 0) && (ix < cols - 1) && (p == img[(iy - 1) * cols + ix + 1]);
            int64_t label = n_w ? iy * cols + ix - 1 : iy * cols + ix;
            if (n_ne) label = (iy - 1) * cols + ix + 1;
            if (n_n) label = (iy - 1) * cols + ix;
            if (n_nw) label = (iy - 1) * cols + ix - 1;
            labels[iy * cols + ix] = (uint32_t)label;
        }
    }
    /* resolve_labels */
    for (int64_t id = 0; id < rows * cols; ++id) labels[id] = find_root(labels, labels[id]);
    /* label_reduction */
    for (iy = 0; iy < rows; ++iy) {
        for (ix = 0; ix < cols; ++ix) {
            float p = img[iy * cols + ix];
            int n_n = (iy > 0) && (p == img[(iy - 1) * cols + ix]);
            if (n_n) continue;
            int n_nw = (iy > 0) && (ix > 0) && (p == img[(iy - 1) * cols + ix - 1]);
            int n_w = (ix > 0) && (p == img[iy * cols + ix - 1]);
            int n_ne = (iy > 0) && (ix < cols - 1) && (p == img[(iy - 1) * cols + ix + 1]);
            if (n_ne) {
                if ((n_nw && n_w) || (n_nw && !n_w))
                    reduction(labels, labels[iy * cols + ix], labels[(iy - 1) * cols + ix + 1]);
                if (!n_nw && n_w)
                    reduction(labels, labels[iy * cols + ix], labels[iy * cols + ix - 1]);
            }
        }
    }
    /* resolve_labels */
    for (int64_t id = 0; id < rows * cols; ++id) labels[id] = find_root(labels, labels[id]);
    /* resolve_background */
    for (int64_t id = 0; id < rows * cols; ++id) labels[id] = (img[id] > 0.0f) ? labels[id] + 1u : 0u;
}
