# ParticleHolographyGB300.jl -- drop-in bodies for ParticleHolography.jl's
# reconstruction hot path (src/holofunc.jl, src/ccl.jl) that forward to
# libphgb300.so through `ccall`.  Same exported names, argument types and
# failure modes (AssertionError / ArgumentError) as the reference.
#
# Julia is not available where this library is built, so this file is not
# exercised by the repository's tests; the same C ABI is exercised from Python
# (ctypes) by tests/ on a GB300.

module ParticleHolographyGB300

using CUDA
using FixedPointNumbers

import ParticleHolography: CuTransferSqrtPart, CuTransfer, CuWavefront, CuLowPassFilter

export cu_transfer_sqrt_arr, cu_transfer, cu_gabor_wavefront, cu_phase_retrieval_holo, cu_get_reconst_vol,
       cu_get_reconst_xyprojection, cu_get_reconst_vol_and_xyprojection, cu_get_reconst_complex_vol,
       cu_asm_prop!, cu_2d_pad, cu_get_reconst_vol_and_xyprojection_padded,
       cu_connected_component_labeling, count_labels, cu_find_valid_labels,
       cu_get_reconst_xyprojection_argmin, cu_get_reconst_xyprojection_range, unpack_projection,
       cu_apply_low_pass_filter!, cu_apply_low_pass_filter,
       cu_rectangle_filter, cu_super_gaussian_filter, cu_get_reconst_xyprojection_lpf,
       cu_get_reconst_binary_vol, slice_bounding_rectangles, cu_reconst_subvolumes,
       cu_make_background_mode, pad_with_mean, autotune!,
       ReconBatch, run!, Server, submit!, poll

const libphgb300 = get(ENV, "PHGB300_LIB", joinpath(@__DIR__, "..", "libphgb300.so"))

const PH_OK = Int32(0)
const PH_ERR_SIZE = Int32(1)
const PH_ERR_DTYPE = Int32(2)
const PH_ERR_TOO_LARGE = Int32(3)
const PH_N0F8, PH_F16, PH_F32, PH_F64, PH_C64, PH_BOOL = Int32.(0:5)

# one context per device, created on first use
const _ctxs = Dict{Int,Ptr{Cvoid}}()
function _ctx()
    dev = CUDA.deviceid(CUDA.device())
    get!(_ctxs, dev) do
        h = Ref{Ptr{Cvoid}}(C_NULL)
        st = ccall((:ph_create, libphgb300), Int32, (Int32, Csize_t, Ref{Ptr{Cvoid}}), dev, 0, h)
        st == PH_OK || error("ph_create failed ($st)")
        h[]
    end
end

_stream() = CUDA.stream().handle

function _check(st::Int32)
    st == PH_OK && return nothing
    msg = unsafe_string(ccall((:ph_last_error, libphgb300), Cstring, (Ptr{Cvoid},), _ctx()))
    st in (PH_ERR_SIZE, PH_ERR_TOO_LARGE) && throw(AssertionError(msg))
    st == PH_ERR_DTYPE && throw(ArgumentError(msg))
    error("libphgb300: $msg (status $st)")
end

const _rt = Dict{Type,Int32}(N0f8 => PH_N0F8, Float16 => PH_F16, Float32 => PH_F32, Float64 => PH_F64)
_rtcode(T) = haskey(_rt, T) ? _rt[T] :
    throw(ArgumentError("return_type must be Subtype of AbstractFloat or N0f8. Got $T"))

# ---- holofunc.jl -----------------------------------------------------------------

function cu_transfer_sqrt_arr(datlen::Int, wavlen::AbstractFloat, dx::AbstractFloat)
    Plane = CuArray{Float32}(undef, datlen, datlen)
    _check(ccall((:ph_transfer_sqrt, libphgb300), Int32,
                 (Ptr{Cvoid}, CuPtr{Float32}, Int32, Int32, Float64, Float64, Ptr{Cvoid}),
                 _ctx(), Plane, datlen, datlen, wavlen, dx, _stream()))
    return CuTransferSqrtPart(Plane)
end

function cu_transfer(z0::AbstractFloat, datLen::Int, wavLen::AbstractFloat, d_sqr::CuTransferSqrtPart{Float32})
    Plane = CuArray{ComplexF32}(undef, datLen, datLen)
    _check(ccall((:ph_transfer, libphgb300), Int32,
                 (Ptr{Cvoid}, CuPtr{ComplexF32}, CuPtr{Float32}, Int32, Int32, Float64, Float64, Ptr{Cvoid}),
                 _ctx(), Plane, d_sqr.data, datLen, datLen, z0, wavLen, _stream()))
    return CuTransfer(Plane)
end

function cu_gabor_wavefront(holo::CuArray{Float32,2})
    out = CuArray{ComplexF32}(undef, size(holo))
    _check(ccall((:ph_gabor_wavefront, libphgb300), Int32,
                 (Ptr{Cvoid}, CuPtr{ComplexF32}, CuPtr{Float32}, Int32, Int32, Ptr{Cvoid}),
                 _ctx(), out, holo, size(holo, 1), size(holo, 2), _stream()))
    return CuWavefront(out)
end

function cu_phase_retrieval_holo(holo1::CuArray{Float32,2}, holo2::CuArray{Float32,2}, transfer::CuTransfer{ComplexF32},
                                 invtransfer::CuTransfer{ComplexF32}, priter::Int, datlen::Int)
    @assert size(holo1) == size(holo2) == size(transfer.data) == size(invtransfer.data) == (datlen, datlen) "All arrays must have the same size as ($datlen, $datlen). Got $(size(holo1)), $(size(holo2)), $(size(transfer.data)), $(size(invtransfer.data))."
    out = CuArray{ComplexF32}(undef, datlen, datlen)
    _check(ccall((:ph_phase_retrieval, libphgb300), Int32,
                 (Ptr{Cvoid}, CuPtr{ComplexF32}, CuPtr{Float32}, CuPtr{Float32}, CuPtr{ComplexF32}, CuPtr{ComplexF32},
                  Int32, Int32, Int32, CuPtr{Float64}, Ptr{Cvoid}),
                 _ctx(), out, holo1, holo2, transfer.data, invtransfer.data, datlen, datlen, priter, CU_NULL, _stream()))
    return CuWavefront(out)
end

function cu_2d_pad(inarr)
    inlen = size(inarr, 1)
    out = CuArray{ComplexF32}(undef, 2 * inlen, 2 * inlen)
    _check(ccall((:ph_pad2d, libphgb300), Int32, (Ptr{Cvoid}, CuPtr{ComplexF32}, CuPtr{ComplexF32}, Int32, Int32, Ptr{Cvoid}),
                 _ctx(), out, inarr, inlen, size(inarr, 2), _stream()))
    return out
end

function _vol(wavefront, transfer_front, transfer_dz, slices, code, T, proj)
    @assert size(wavefront.data) == size(transfer_front.data) == size(transfer_dz.data) "All arrays must have the same size. Got $(size(wavefront.data)), $(size(transfer_front.data)), $(size(transfer_dz.data))."
    vol = CuArray{T}(undef, size(wavefront.data)..., slices)
    _check(ccall((:ph_reconst_vol, libphgb300), Int32,
                 (Ptr{Cvoid}, CuPtr{Cvoid}, Int32, CuPtr{Float32}, CuPtr{ComplexF32}, CuPtr{ComplexF32},
                  CuPtr{ComplexF32}, Int32, Int32, Int32, Ptr{Cvoid}),
                 _ctx(), vol, code, proj === nothing ? CU_NULL : proj, wavefront.data, transfer_front.data,
                 transfer_dz.data, size(wavefront.data, 1), size(wavefront.data, 2), slices, _stream()))
    return vol
end

cu_get_reconst_vol(wavefront::CuWavefront{ComplexF32}, transfer_front::CuTransfer{ComplexF32},
                   transfer_dz::CuTransfer{ComplexF32}, slices::Int, return_type::Type=N0f8) =
    _vol(wavefront, transfer_front, transfer_dz, slices, _rtcode(return_type), return_type, nothing)

cu_get_reconst_complex_vol(wavefront::CuWavefront{ComplexF32}, transfer_front::CuTransfer{ComplexF32},
                           transfer_dz::CuTransfer{ComplexF32}, slices::Int) =
    _vol(wavefront, transfer_front, transfer_dz, slices, PH_C64, ComplexF32, nothing)

function cu_get_reconst_vol_and_xyprojection(wavefront::CuWavefront{ComplexF32}, transfer_front::CuTransfer{ComplexF32},
                                             transfer_dz::CuTransfer{ComplexF32}, slices::Int, return_type::Type=N0f8)
    proj = CuArray{Float32}(undef, size(wavefront.data)...)
    vol = _vol(wavefront, transfer_front, transfer_dz, slices, _rtcode(return_type), return_type, proj)
    return vol, proj
end

function _xyproj(wavefront, transfer_front, transfer_dz, slices, argmin)
    @assert size(wavefront.data) == size(transfer_front.data) == size(transfer_dz.data) "All arrays must have the same size. Got $(size(wavefront.data)), $(size(transfer_front.data)), $(size(transfer_dz.data))."
    proj = CuArray{Float32}(undef, size(wavefront.data)...)
    _check(ccall((:ph_reconst_xyproj, libphgb300), Int32,
                 (Ptr{Cvoid}, CuPtr{Float32}, CuPtr{Int32}, CuPtr{ComplexF32}, CuPtr{ComplexF32}, CuPtr{ComplexF32},
                  Int32, Int32, Int32, Ptr{Cvoid}),
                 _ctx(), proj, argmin === nothing ? CU_NULL : argmin, wavefront.data, transfer_front.data,
                 transfer_dz.data, size(wavefront.data, 1), size(wavefront.data, 2), slices, _stream()))
    return proj
end

cu_get_reconst_xyprojection(wavefront::CuWavefront{ComplexF32}, transfer_front::CuTransfer{ComplexF32},
                            transfer_dz::CuTransfer{ComplexF32}, slices::Int) =
    _xyproj(wavefront, transfer_front, transfer_dz, slices, nothing)

"New: the projection and the 1-based slice index of its first minimum."
function cu_get_reconst_xyprojection_argmin(wavefront::CuWavefront{ComplexF32}, transfer_front::CuTransfer{ComplexF32},
                                            transfer_dz::CuTransfer{ComplexF32}, slices::Int)
    arg = CuArray{Int32}(undef, size(wavefront.data)...)
    proj = _xyproj(wavefront, transfer_front, transfer_dz, slices, arg)
    return proj, arg .+ Int32(1)
end

"""New: one depth shard of `cu_get_reconst_xyprojection`, slices `k0:k1-1`
(0-based, global) reduced to packed words `(Float32 bits << 32) | slice`.
Merge the shards of a frame with `min.` (or an `Int64` MIN all-reduce across
GPUs) and unpack them with `unpack_projection`."""
function cu_get_reconst_xyprojection_range(wavefront::CuWavefront{ComplexF32}, transfer_front::CuTransfer{ComplexF32},
                                           transfer_dz::CuTransfer{ComplexF32}, k0::Int, k1::Int;
                                           packed::Union{CuArray{Int64,2},Nothing}=nothing, accumulate::Bool=false)
    @assert size(wavefront.data) == size(transfer_front.data) == size(transfer_dz.data) "All arrays must have the same size. Got $(size(wavefront.data)), $(size(transfer_front.data)), $(size(transfer_dz.data))."
    out = packed === nothing ? CuArray{Int64}(undef, size(wavefront.data)...) : packed
    _check(ccall((:ph_reconst_xyproj_range, libphgb300), Int32,
                 (Ptr{Cvoid}, CuPtr{Int64}, CuPtr{ComplexF32}, CuPtr{ComplexF32}, CuPtr{ComplexF32},
                  Int32, Int32, Int32, Int32, Int32, Ptr{Cvoid}),
                 _ctx(), out, wavefront.data, transfer_front.data, transfer_dz.data, size(wavefront.data, 1),
                 size(wavefront.data, 2), k0, k1, accumulate ? Int32(1) : Int32(0), _stream()))
    return out
end

"New: merged packed words -> (projection, 1-based slice index of the first minimum)."
function unpack_projection(packed::CuArray{Int64,2})
    proj = CuArray{Float32}(undef, size(packed)...)
    arg = CuArray{Int32}(undef, size(packed)...)
    _check(ccall((:ph_unpack_projection, libphgb300), Int32,
                 (Ptr{Cvoid}, CuPtr{Float32}, CuPtr{Int32}, CuPtr{Int64}, Int32, Int32, Ptr{Cvoid}),
                 _ctx(), proj, arg, packed, size(packed, 1), size(packed, 2), _stream()))
    return proj, arg .+ Int32(1)
end

function cu_get_reconst_vol_and_xyprojection_padded(wavefront::CuWavefront{ComplexF32}, transfer_front::CuTransfer{ComplexF32},
                                                    transfer_dz::CuTransfer{ComplexF32}, slices::Int, return_type::Type=N0f8)
    expected_size = map(x -> 2 * x, size(wavefront.data))
    @assert expected_size == size(transfer_front.data) == size(transfer_dz.data) "size(transfer_front.data) and size(transfer_dz.data) must be equal to 2*size(wavefront.data). Got $(size(wavefront.data)), $(size(transfer_front.data)), $(size(transfer_dz.data))."
    datlen = size(wavefront.data, 1)
    vol = CuArray{N0f8}(undef, datlen, datlen, slices)
    proj = CuArray{Float32}(undef, datlen, datlen)
    _check(ccall((:ph_reconst_vol_padded, libphgb300), Int32,
                 (Ptr{Cvoid}, CuPtr{N0f8}, CuPtr{Float32}, CuPtr{ComplexF32}, CuPtr{ComplexF32}, CuPtr{ComplexF32},
                  Int32, Int32, Int32, Int32, Ptr{Cvoid}),
                 _ctx(), vol, proj, wavefront.data, transfer_front.data, transfer_dz.data, datlen,
                 size(wavefront.data, 2), slices, _rtcode(return_type), _stream()))
    return vol, proj
end

function cu_asm_prop!(outholo::CuWavefront, inholo::CuWavefront, d_sqr::CuTransferSqrtPart, zprop::Float64, datlen::Int,
                      λ::Float64)
    _check(ccall((:ph_asm_prop, libphgb300), Int32,
                 (Ptr{Cvoid}, CuPtr{ComplexF32}, CuPtr{ComplexF32}, CuPtr{Float32}, Float64, Int32, Int32, Float64,
                  Ptr{Cvoid}),
                 _ctx(), outholo.data, inholo.data, d_sqr.data, zprop, datlen, datlen, λ, _stream()))
    return nothing
end

# ---- frequency_filters.jl ---------------------------------------------------------

function cu_apply_low_pass_filter!(holo::CuWavefront, lpf::CuLowPassFilter)
    _check(ccall((:ph_apply_lpf, libphgb300), Int32,
                 (Ptr{Cvoid}, CuPtr{ComplexF32}, CuPtr{ComplexF32}, CuPtr{Float32}, Int32, Int32, Ptr{Cvoid}),
                 _ctx(), holo.data, holo.data, lpf.data, size(holo.data, 1), size(holo.data, 2), _stream()))
    return nothing
end

function cu_apply_low_pass_filter(holo::CuWavefront, lpf::CuLowPassFilter)
    out = CuWavefront(copy(holo.data))
    cu_apply_low_pass_filter!(out, lpf)
    return out
end

# ---- ccl.jl ------------------------------------------------------------------------

function cu_connected_component_labeling(input_img)
    @assert length(input_img) <= 2^32 - 1 "Image is too large. Maximum length is 2^32-1."
    output_img = CuArray{UInt32}(undef, size(input_img))
    height, width = size(input_img)
    code = eltype(input_img) == Bool ? PH_BOOL : PH_F32
    img = eltype(input_img) in (Bool, Float32) ? input_img : Float32.(input_img)
    _check(ccall((:ph_ccl, libphgb300), Int32,
                 (Ptr{Cvoid}, CuPtr{UInt32}, CuPtr{Cvoid}, Int32, Int64, Int64, Ptr{Cvoid}),
                 _ctx(), output_img, img, code, height, width, _stream()))   # the reference's grid: rows = size(img,1)
    return output_img
end

function _roots(labels::CuArray{UInt32}, capacity::Int)
    roots = Vector{Int64}(undef, capacity)
    count = Ref{Int64}(0)
    _check(ccall((:ph_ccl_roots, libphgb300), Int32,
                 (Ptr{Cvoid}, Ptr{Int64}, Int64, Ref{Int64}, CuPtr{UInt32}, Int64, Ptr{Cvoid}),
                 _ctx(), roots, capacity, count, labels, length(labels), _stream()))
    return count[], roots
end

count_labels(labels::CuArray{UInt32}) = _roots(labels, 0)[1]
count_labels(labels::Array{UInt32}) = count_labels(CuArray(labels))

function cu_find_valid_labels(labels::CuArray{UInt32,2})
    c, _ = _roots(labels, 0)
    _, roots = _roots(labels, c)
    return roots[1:c]
end

# ---- frequency_filters.jl ------------------------------------------------------------

for (name, sym) in ((:cu_rectangle_filter, :ph_lpf_rectangle), (:cu_super_gaussian_filter, :ph_lpf_super_gaussian))
    @eval function $name(prop_dist::AbstractFloat, wavlen::AbstractFloat, imglen::Int, pixel_picth::AbstractFloat)
        arr = CuArray{Float32}(undef, imglen, imglen)
        _check(ccall(($(QuoteNode(sym)), libphgb300), Int32,
                     (Ptr{Cvoid}, CuPtr{Float32}, Int32, Float64, Float64, Float64, Ptr{Cvoid}),
                     _ctx(), arr, imglen, prop_dist, wavlen, pixel_picth, _stream()))
        return CuLowPassFilter(arr)
    end
end

# cu_apply_low_pass_filter then cu_get_reconst_xyprojection, the filter folded into
# the spectrum (no FFT pair); also returns the argmin depth (0-based, Int32).
function cu_get_reconst_xyprojection_lpf(light_field::CuWavefront{ComplexF32}, transfer_front::CuTransfer{ComplexF32},
                                         transfer_dz::CuTransfer{ComplexF32}, lpf::CuLowPassFilter, slices::Int)
    n1, n2 = size(light_field.data)
    @assert size(transfer_front.data) == size(transfer_dz.data) == size(lpf.data) == (n1, n2) "All arrays must have the same size."
    proj = CuArray{Float32}(undef, n1, n2)
    amin = CuArray{Int32}(undef, n1, n2)
    _check(ccall((:ph_reconst_xyproj_lpf, libphgb300), Int32,
                 (Ptr{Cvoid}, CuPtr{Float32}, CuPtr{Int32}, CuPtr{ComplexF32}, CuPtr{ComplexF32}, CuPtr{ComplexF32},
                  CuPtr{Float32}, Int32, Int32, Int32, Ptr{Cvoid}),
                 _ctx(), proj, amin, light_field.data, transfer_front.data, transfer_dz.data, lpf.data, n1, n2, slices,
                 _stream()))
    return proj, amin
end

# ---- particle_detection.jl (the device side of particle_bounding_boxes) ----------------

# cu_get_reconst_vol(..., Float32) .<= threshold in one pass, without the Float32 volume.
function cu_get_reconst_binary_vol(light_field::CuWavefront{ComplexF32}, transfer_front::CuTransfer{ComplexF32},
                                   transfer_dz::CuTransfer{ComplexF32}, slices::Int, threshold::Real)
    n1, n2 = size(light_field.data)
    @assert size(transfer_front.data) == size(transfer_dz.data) == (n1, n2) "All arrays must have the same size."
    vol = CuArray{Bool}(undef, n1, n2, slices)
    _check(ccall((:ph_reconst_binary_vol, libphgb300), Int32,
                 (Ptr{Cvoid}, CuPtr{Bool}, Float32, CuPtr{Float32}, CuPtr{ComplexF32}, CuPtr{ComplexF32},
                  CuPtr{ComplexF32}, Int32, Int32, Int32, Ptr{Cvoid}),
                 _ctx(), vol, threshold, CU_NULL, light_field.data, transfer_front.data, transfer_dz.data, n1, n2,
                 slices, _stream()))
    return vol
end

# For every slice of a binary volume, what
# get_bounding_rectangles(Array(cu_connected_component_labeling(vol[:, :, k])),
#                         cu_find_valid_labels(...))
# returns, (x_min, y_min, x_max, y_max) per component in root order: all slices
# labelled in one launch set and boxed on the device.  The loop of
# particle_bounding_boxes then only merges neighbourhoods on the host.
function slice_bounding_rectangles(d_bin_vol::CuArray{Bool,3})
    rows, cols, slices = size(d_bin_vol)
    labels = CuArray{UInt32}(undef, rows, cols, slices)
    _check(ccall((:ph_ccl_batch, libphgb300), Int32,
                 (Ptr{Cvoid}, CuPtr{UInt32}, CuPtr{Cvoid}, Int32, Int64, Int64, Int64, Ptr{Cvoid}),
                 _ctx(), labels, d_bin_vol, PH_BOOL, slices, rows, cols, _stream()))
    count = Ref{Int64}(0)
    boxes_call(buf, cap) = _check(ccall((:ph_ccl_boxes, libphgb300), Int32,
                                        (Ptr{Cvoid}, Ptr{Int64}, Int64, Ref{Int64}, CuPtr{UInt32}, Int64, Int64, Int64,
                                         Ptr{Cvoid}),
                                        _ctx(), buf, cap, count, labels, slices, rows, cols, _stream()))
    boxes_call(C_NULL, 0)
    boxes = Vector{Int64}(undef, 5 * count[])
    boxes_call(boxes, count[])
    out = [NTuple{4,Int}[] for _ in 1:slices]
    per = rows * cols
    for b in 1:count[]
        root, x0, y0, x1, y1 = boxes[5b-4], boxes[5b-3], boxes[5b-2], boxes[5b-1], boxes[5b]
        push!(out[div(root - 1, per) + 1], (x0, y0, x1, y1))
    end
    return out
end

# The N0f8 sub-volumes particle_coordinates / particle_coor_diams cut out of
# cu_get_reconst_vol(..., N0f8): d_vol[y_min:y_max, x_min:x_max, z_min:z_max] for
# each box (x_min, y_min, z_min, x_max, y_max, z_max) (particle_bbs order,
# 1-based inclusive), without the volume; only the covered slices are computed.
function cu_reconst_subvolumes(light_field::CuWavefront{ComplexF32}, transfer_front::CuTransfer{ComplexF32},
                               transfer_dz::CuTransfer{ComplexF32}, slices::Int, boxes::AbstractVector)
    n1, n2 = size(light_field.data)
    @assert size(transfer_front.data) == size(transfer_dz.data) == (n1, n2) "All arrays must have the same size."
    n = length(boxes)
    bx = Vector{Int64}(undef, 6n)
    for (i, b) in enumerate(boxes)
        bx[6i-5:6i] .= Int64.(collect(b))
    end
    offs = zeros(Int64, n + 1)
    sub(out, wf, tf, td) = _check(ccall((:ph_reconst_subvolumes, libphgb300), Int32,
                                        (Ptr{Cvoid}, CuPtr{UInt8}, Ptr{Int64}, Ptr{Int64}, Int32, CuPtr{ComplexF32},
                                         CuPtr{ComplexF32}, CuPtr{ComplexF32}, Int32, Int32, Int32, Ptr{Cvoid}),
                                        _ctx(), out, offs, bx, n, wf, tf, td, n1, n2, slices, _stream()))
    sub(CU_NULL, CU_NULL, CU_NULL, CU_NULL)   # sizes only
    out = CuArray{UInt8}(undef, max(offs[end], 1))
    n > 0 && sub(out, light_field.data, transfer_front.data, transfer_dz.data)
    return [reinterpret(N0f8, reshape(out[offs[i]+1:offs[i+1]], b[5] - b[2] + 1, b[4] - b[1] + 1, b[6] - b[3] + 1))
            for (i, b) in enumerate(boxes)]
end

# ---- utils.jl ------------------------------------------------------------------------

# Per-pixel mode of the images (the first maximum on ties) / 255, on the host as
# the reference returns it; images not already UInt8 are scaled by 255 and rounded.
function cu_make_background_mode(grayimglist)
    H, W = size(grayimglist[1])
    imgs = CuArray{UInt8}(undef, H, W, length(grayimglist))
    for (k, img) in enumerate(grayimglist)
        u8 = eltype(img) === UInt8 ? img : map(v -> UInt8(round(clamp(Float32(v) * 255f0, 0f0, 255f0))), img)
        copyto!(view(imgs, :, :, k), u8)
    end
    out = CuArray{Float64}(undef, H, W)
    _check(ccall((:ph_background_mode, libphgb300), Int32,
                 (Ptr{Cvoid}, CuPtr{Float64}, CuPtr{UInt8}, Int64, Int32, Int32, Ptr{Cvoid}),
                 _ctx(), out, imgs, length(grayimglist), H, W, _stream()))
    return Array(out)
end

function pad_with_mean(img::CuArray{Float32,2}, padsize::Int)
    @assert padsize > size(img, 1) && padsize > size(img, 2) "Padsize should be larger than the image size. padsize: $padsize, img size: $(size(img))"
    out = CuArray{Float32}(undef, padsize, padsize)
    _check(ccall((:ph_pad_with_mean, libphgb300), Int32,
                 (Ptr{Cvoid}, CuPtr{Float32}, CuPtr{Float32}, Int32, Int32, Int32, Ptr{Cvoid}),
                 _ctx(), out, img, size(img, 1), size(img, 2), padsize, _stream()))
    return out
end
pad_with_mean(img::Array{Float32,2}, padsize::Int) = Array(pad_with_mean(CuArray(img), padsize))

# ---- batches and serving (no single reference counterpart) ------------------------

# ph_recon_item (phgb300.h)
struct _ReconItem
    hologram::CuPtr{Float32}
    wavefront::CuPtr{ComplexF32}
    tf_front::CuPtr{ComplexF32}
    tf_dz::CuPtr{ComplexF32}
    proj::CuPtr{Float32}
    argmin::CuPtr{Int32}
    n_fast::Int32
    n_slow::Int32
    slices::Int32
end

# A batch of cu_get_reconst_xyprojection calls (holofunc.jl:248-266) recorded as
# one CUDA graph; `items` are (hologram::CuArray{Float32,2}, transfer_front,
# transfer_dz, slices) tuples.  The arrays must outlive the batch.
mutable struct ReconBatch
    handle::Ptr{Cvoid}
    proj::Vector{CuArray{Float32,2}}
    argmin::Vector{CuArray{Int32,2}}
    keep::Vector{Any}
end

function ReconBatch(items; lanes::Int=4)
    recs = _ReconItem[]
    proj = CuArray{Float32,2}[]
    amin = CuArray{Int32,2}[]
    for (holo, tf, td, slices) in items
        @assert size(holo) == size(tf.data) == size(td.data) "All arrays must have the same size. Got $(size(holo)), $(size(tf.data)), $(size(td.data))."
        p = CuArray{Float32}(undef, size(holo)...)
        a = CuArray{Int32}(undef, size(holo)...)
        push!(proj, p); push!(amin, a)
        push!(recs, _ReconItem(pointer(holo), CU_NULL, pointer(tf.data), pointer(td.data), pointer(p), pointer(a),
                               size(holo, 1), size(holo, 2), slices))
    end
    CUDA.synchronize()
    h = Ref{Ptr{Cvoid}}(C_NULL)
    _check(ccall((:ph_batch_plan, libphgb300), Int32, (Ptr{Cvoid}, Ptr{_ReconItem}, Int32, Int32, Ref{Ptr{Cvoid}}),
                 _ctx(), recs, length(recs), lanes, h))
    b = ReconBatch(h[], proj, amin, Any[items])
    finalizer(b) do x
        x.handle == C_NULL || ccall((:ph_batch_destroy, libphgb300), Cvoid, (Ptr{Cvoid},), x.handle)
    end
    return b
end

function run!(b::ReconBatch)
    _check(ccall((:ph_batch_run, libphgb300), Int32, (Ptr{Cvoid}, Ptr{Cvoid}), b.handle, _stream()))
    return b.proj, b.argmin
end

"""New: times the reconstruction knobs of one shape once (slices per CTA, batch of
intermediates and, with `allow_forms`, the split-precision row-pass forms) and
keeps the fastest for later calls, batches and servers; `cache` is a JSON file
keyed by device and shape.  Returns (form, group cap, batch slices, ms)."""
function autotune!(n_fast::Int, n_slow::Int, slices::Int; allow_forms::Bool=false,
                   cache::Union{Nothing,String}=nothing)
    choice = zeros(Int32, 3)
    ms = Ref{Float64}(0.0)
    path = cache === nothing ? nothing : Base.cconvert(Cstring, cache)   # NUL-terminated, kept alive below
    GC.@preserve path begin
        _check(ccall((:ph_autotune, libphgb300), Int32,
                     (Ptr{Cvoid}, Int32, Int32, Int32, Int32, Ptr{UInt8}, Ptr{Int32}, Ref{Float64}, Ptr{Cvoid}),
                     _ctx(), n_fast, n_slow, slices, allow_forms ? Int32(1) : Int32(0),
                     path === nothing ? Ptr{UInt8}(C_NULL) : pointer(path), choice, ms, _stream()))
    end
    return (Int(choice[1]), Int(choice[2]), Int(choice[3]), ms[])
end

# ph_serve_request (phgb300.h)
struct _ServeRequest
    hologram::CuPtr{Float32}
    proj::CuPtr{Float32}
    argmin::CuPtr{Int32}
    n_fast::Int32
    n_slow::Int32
    slices::Int32
    z0::Float64
    dz::Float64
    wavlen::Float64
    dx::Float64
    frame::CuPtr{UInt8}          # device ingest of an 8-bit frame (CU_NULL: use hologram)
    frame_n_fast::Int32
    frame_n_slow::Int32
    frame_pitch::Int32
    frame_channels::Int32
    frame_flip::Int32
    background::CuPtr{Float64}
    background_offset::Float64
end

mutable struct Server
    handle::Ptr{Cvoid}
    live::Dict{Int64,Any}
end

function Server(max_size::Tuple{Int,Int}, max_slices::Int; lanes::Int=3, tf_cache::Int=16, budget::Integer=0)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    _check(ccall((:ph_serve_create, libphgb300), Int32,
                 (Ptr{Cvoid}, Int32, Int32, Int32, Int32, Int32, Csize_t, Ref{Ptr{Cvoid}}),
                 _ctx(), lanes, max_size[1], max_size[2], max_slices, tf_cache, budget, h))
    s = Server(h[], Dict{Int64,Any}())
    finalizer(s) do x
        x.handle == C_NULL || ccall((:ph_serve_destroy, libphgb300), Cvoid, (Ptr{Cvoid},), x.handle)
    end
    return s
end

# Queues the projection of `holo` into `proj` (and `argmin`); returns a ticket.
function submit!(s::Server, holo::CuArray{Float32,2}, proj::CuArray{Float32,2}, slices::Int, z0::Real, dz::Real;
                 wavlen::Real=0.6328, dx::Real=10.0, argmin::Union{Nothing,CuArray{Int32,2}}=nothing)
    req = Ref(_ServeRequest(pointer(holo), pointer(proj), argmin === nothing ? CU_NULL : pointer(argmin),
                            size(holo, 1), size(holo, 2), slices, z0, dz, wavlen, dx,
                            CU_NULL, 0, 0, 0, 0, 0, CU_NULL, 0.0))
    t = Ref{Int64}(0)
    _check(ccall((:ph_serve_submit, libphgb300), Int32, (Ptr{Cvoid}, Ref{_ServeRequest}, Ref{Int64}, Ptr{Cvoid}),
                 s.handle, req, t, _stream()))
    s.live[t[]] = (holo, proj, argmin)
    return t[]
end

# The request's latency in ms once finished, `nothing` while pending.
function poll(s::Server, ticket::Int64; wait::Bool=false)
    lat = Ref{Float64}(0.0)
    st = ccall((:ph_serve_poll, libphgb300), Int32, (Ptr{Cvoid}, Int64, Int32, Ref{Float64}), s.handle, ticket,
               wait ? 1 : 0, lat)
    st == Int32(9) && return nothing
    _check(st)
    delete!(s.live, ticket)
    return lat[]
end

end # module
