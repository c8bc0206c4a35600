# BlueTangleGPU: GPU-resident states for BlueTangle.jl through libbtgpu (C ABI,
# include/btgpu.h).  BlueTangle reaches its hot path through multiple dispatch on
# the state argument (apply, measure, sample, expect, correlation, born_measure_Z,
# fidelity: src/BlueTangle.jl:5-22); this module adds methods of those generics for
# GPU handles.  Matrices and Kraus sets still come from BlueTangle's own
# constructors (op.mat, op.kraus, noise.q1.kraus), so the values are the
# reference's.
#
# Every method follows the Python host mirror of the same entry points
# (bluetangle_gpu/engine.py, trajectories.py), which the test suite runs against
# the oracle on a GPU: the same ABI calls with the same arguments, in the same
# order.  `apply` is functional as in the reference (src/hilbert.jl:505, :514: it
# returns a new state and leaves its argument as it was); `apply!` is the in-place
# form the mirror's `apply` is.
#
#   using BlueTangle, BlueTangleGPU
#   psi = gpu_zero_state(20)                     # |0...0>, complex128
#   psi2 = apply(psi, [Op("H", 1), Op("CNOT", 1, 2)]; noise=NoiseModel("depolarizing", 0.01))
#   expect(psi2, "Z")
module BlueTangleGPU

using BlueTangle
using LinearAlgebra
import BlueTangle: apply, sample, sample_exact, expect, correlation, born_measure_Z, measure, fidelity,
                   apply_noise, get_N

export GPUContext, GPUState, GPUDensity, GPUPlan, GPUProgram, GPUServer, BTError
export gpu_zero_state, gpu_zero_rho, gpu_state, gpu_rho, apply!, born_measure_Z!, apply_noise!
export gpu_compile, gpu_compile_variational, run!, run_members!, set_matrices!, plan_cost
export gpu_shots, gpu_shot_samples, gpu_measure, gpu_product_state, add_client, submit, result, serve_stats
export gpu_variational_apply, gpu_loss, gpu_loss_and_grad_paramshift, gpu_shadow
export gpu_to_state, gpu_to_rho, gpu_run, gpu_one_state, gpu_neel_state01, gpu_neel_state10, gpu_Z3, gpu_Z3_s,
       gpu_neel_state_s, gpu_plus_state, gpu_minus_state, gpu_random_product_state, gpu_random_state

# the library: BTGPU_LIB, else the in-tree build next to this directory
const lib = get(ENV, "BTGPU_LIB", joinpath(@__DIR__, "..", "bluetangle.jl_gb300", "libbtgpu.so"))

const BT_REPR_SV, BT_REPR_DM = Cint(0), Cint(1)
const BT_PREC_C128, BT_PREC_C64 = Cint(0), Cint(1)
const BT_KRAUS_TRAJ, BT_KRAUS_SUM = Cint(0), Cint(1)
const BT_KRAUS_REF_ORDER, BT_KRAUS_UNITARY_MIX = Cint(0x100), Cint(0x200)
const PRECISIONS = Dict(:c128 => BT_PREC_C128, :c64 => BT_PREC_C64)

# ------------------------------------------------------------------ errors
"""Status of a failed call and the library's message (bt_last_error)."""
struct BTError <: Exception
    code::Int
    msg::String
end
Base.showerror(io::IO, e::BTError) = print(io, e.msg, " (status ", e.code, ")")

function check(rc::Cint, ctx::Ptr{Cvoid})
    rc == 0 && return nothing
    p = ccall((:bt_last_error, lib), Cstring, (Ptr{Cvoid},), ctx)
    msg = p == C_NULL ? unsafe_string(ccall((:bt_status_string, lib), Cstring, (Cint,), rc)) : unsafe_string(p)
    throw(BTError(Int(rc), msg))
end

# ------------------------------------------------------------------ context
"""One CUDA device and stream (bt_ctx)."""
mutable struct GPUContext
    h::Ptr{Cvoid}
end
function GPUContext(device::Integer=0; seed::Integer=0x5EED)
    r = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:bt_ctx_create, lib), Cint, (Cint, UInt64, Ptr{Ptr{Cvoid}}), device, seed % UInt64, r), C_NULL)
    c = GPUContext(r[])
    finalizer(c) do x
        x.h != C_NULL && ccall((:bt_ctx_destroy, lib), Cint, (Ptr{Cvoid},), x.h)
        x.h = C_NULL
    end
    return c
end
const _default_ctx = Ref{Union{Nothing,GPUContext}}(nothing)
default_context() = (_default_ctx[] === nothing && (_default_ctx[] = GPUContext()); _default_ctx[])
synchronize(c::GPUContext) = check(ccall((:bt_ctx_synchronize, lib), Cint, (Ptr{Cvoid},), c.h), c.h)
function launch_count(c::GPUContext)
    v = Ref{Int64}(0)
    check(ccall((:bt_ctx_launch_count, lib), Cint, (Ptr{Cvoid}, Ref{Int64}), c.h, v), c.h)
    return v[]
end

# ------------------------------------------------------------------ states
abstract type GPUHandle end

"""2^N amplitudes per member on the GPU (replaces the reference's SparseVector);
`batch` members: trajectories, copies, shots."""
mutable struct GPUState <: GPUHandle
    ctx::GPUContext
    h::Ptr{Cvoid}
    n::Int
    prec::Cint
    batch::Int
end

"""4^N entries per member (replaces SparseMatrixCSC); rho[i, j] lives at i + j 2^N."""
mutable struct GPUDensity <: GPUHandle
    ctx::GPUContext
    h::Ptr{Cvoid}
    n::Int
    prec::Cint
    batch::Int
end

repr_code(::Type{GPUState}) = BT_REPR_SV
repr_code(::Type{GPUDensity}) = BT_REPR_DM

function _free!(s::GPUHandle)
    if s.h != C_NULL && s.ctx.h != C_NULL
        ccall((:bt_state_free, lib), Cint, (Ptr{Cvoid},), s.h)
    end
    s.h = C_NULL
    return nothing
end

function _alloc(::Type{T}, n::Integer, prec::Symbol, batch::Integer, ctx::GPUContext) where {T<:GPUHandle}
    r = Ref{Ptr{Cvoid}}(C_NULL)
    pc = PRECISIONS[prec]
    check(ccall((:bt_state_alloc, lib), Cint, (Ptr{Cvoid}, Cint, Cint, Cint, Cint, Ptr{Ptr{Cvoid}}),
                ctx.h, n, repr_code(T), pc, batch, r), ctx.h)
    return finalizer(_free!, T(ctx, r[], Int(n), pc, Int(batch)))
end

get_N(s::GPUHandle) = s.n
entries(s::GPUHandle) = 1 << (s isa GPUState ? s.n : 2 * s.n)
_prec_symbol(s::GPUHandle) = s.prec == BT_PREC_C64 ? :c64 : :c128

"""zero_state(N) (src/hilbert.jl:866) on the GPU: every member |0...0>."""
gpu_zero_state(N::Integer; prec::Symbol=:c128, batch::Integer=1, ctx::GPUContext=default_context()) =
    _alloc(GPUState, N, prec, batch, ctx)

"""zero_state(N) * zero_state(N)' as a GPU density matrix."""
gpu_zero_rho(N::Integer; prec::Symbol=:c128, batch::Integer=1, ctx::GPUContext=default_context()) =
    _alloc(GPUDensity, N, prec, batch, ctx)

function _upload!(s::GPUHandle, flat::Vector{ComplexF64}, member::Integer)
    length(flat) == entries(s) || throw(ArgumentError("array size does not match the state"))
    check(ccall((:bt_state_upload, lib), Cint, (Ptr{Cvoid}, Int64, Int64, Int64, Ptr{ComplexF64}),
                s.h, member, 0, length(flat), flat), s.ctx.h)
    return s
end

function _download(s::GPUHandle, member::Integer)
    out = Vector{ComplexF64}(undef, entries(s))
    check(ccall((:bt_state_download, lib), Cint, (Ptr{Cvoid}, Int64, Int64, Int64, Ptr{ComplexF64}),
                s.h, member, 0, length(out), out), s.ctx.h)
    return out
end

"""A host state vector (dense or sparse) on the GPU."""
function gpu_state(psi::AbstractVector; prec::Symbol=:c128, ctx::GPUContext=default_context())
    n = round(Int, log2(length(psi)))
    return _upload!(_alloc(GPUState, n, prec, 1, ctx), Vector{ComplexF64}(psi), 0)
end

"""A host density matrix on the GPU (column-major: Julia's own layout)."""
function gpu_rho(rho::AbstractMatrix; prec::Symbol=:c128, ctx::GPUContext=default_context())
    n = round(Int, log2(size(rho, 1)))
    return _upload!(_alloc(GPUDensity, n, prec, 1, ctx), vec(Matrix{ComplexF64}(rho)), 0)
end

Base.Vector(s::GPUState; member::Integer=0) = _download(s, member)
Base.Matrix(s::GPUDensity; member::Integer=0) = reshape(_download(s, member), 1 << s.n, 1 << s.n)

function set_zero!(s::GPUHandle; member::Integer=-1)
    check(ccall((:bt_state_set_zero, lib), Cint, (Ptr{Cvoid}, Int64), s.h, member), s.ctx.h)
    return s
end

function set_basis!(s::GPUHandle, index::Integer; member::Integer=-1)
    check(ccall((:bt_state_set_basis, lib), Cint, (Ptr{Cvoid}, Int64, UInt64), s.h, member, index % UInt64), s.ctx.h)
    return s
end

function copy_from!(dst::GPUHandle, src::GPUHandle; dst_member::Integer=-1, src_member::Integer=0)
    check(ccall((:bt_state_copy, lib), Cint, (Ptr{Cvoid}, Int64, Ptr{Cvoid}, Int64),
                dst.h, dst_member, src.h, src_member), dst.ctx.h)
    return dst
end

"""A new handle holding the same members (bt_state_alloc + bt_state_copy)."""
function Base.copy(s::T) where {T<:GPUHandle}
    c = _alloc(T, s.n, _prec_symbol(s), s.batch, s.ctx)
    for m in 0:s.batch-1
        copy_from!(c, s; dst_member=m, src_member=m)
    end
    return c
end

# the basis index of a list of qubit values, qubit 1 the most significant bit:
# _bin2state(Int(sign(x))) is |0> for 0 and |1> otherwise (src/bit.jl:59)
_basis_index(bits) = foldl((a, b) -> (a << 1) | UInt64(sign(b) != 0), bits; init=UInt64(0))

"""product_state(list_of_qubits) (src/hilbert.jl:835): the basis state of the
bits (qubit 1 the most significant; every non-zero entry is |1>)."""
function gpu_product_state(bits::AbstractVector{<:Real}; prec::Symbol=:c128, ctx::GPUContext=default_context())
    length(bits) <= 64 || throw(ArgumentError("at most 64 qubits"))
    s = _alloc(GPUState, length(bits), prec, 1, ctx)
    return set_basis!(s, _basis_index(bits))
end

"""one_state(N) (src/hilbert.jl:867): |1...1>."""
gpu_one_state(N::Integer; prec::Symbol=:c128, ctx::GPUContext=default_context()) =
    set_basis!(_alloc(GPUState, N, prec, 1, ctx), (UInt64(1) << N) - 1)

"""neel_state01(N), neel_state10(N) (src/hilbert.jl:837-838)."""
gpu_neel_state01(N::Integer; kw...) = gpu_product_state([isodd(i) ? 0 : 1 for i in 1:N]; kw...)
gpu_neel_state10(N::Integer; kw...) = gpu_product_state([isodd(i) ? 1 : 0 for i in 1:N]; kw...)

_z3_bits(N, j) = [mod(i + 2 - j + 1, 3) == 0 ? 1 : 0 for i in 1:N]

"""Z3(N, j) (src/hilbert.jl:844)."""
gpu_Z3(N::Integer, j::Integer=1; kw...) = gpu_product_state(_z3_bits(N, j); kw...)

"""random_product_state(N) = product_state(rand([0, 1], N)) (src/hilbert.jl:859)."""
gpu_random_product_state(N::Integer; kw...) = gpu_product_state(rand([0, 1], N); kw...)

# normalize(sum of the basis states of indices): the state cleared, then each
# distinct index written with its count over the norm
function _superpose(N, indices, prec, ctx)
    s = _alloc(GPUState, N, prec, 1, ctx)
    check(ccall((:bt_state_clear, lib), Cint, (Ptr{Cvoid}, Int64), s.h, 0), ctx.h)
    counts = Dict{UInt64,Float64}()
    for i in indices
        counts[i] = get(counts, i, 0.0) + 1.0
    end
    nrm = sqrt(sum(v^2 for v in values(counts)))
    for (i, v) in counts
        a = ComplexF64[v / nrm]
        check(ccall((:bt_state_upload, lib), Cint, (Ptr{Cvoid}, Int64, Int64, Int64, Ptr{ComplexF64}),
                    s.h, 0, Int64(i), 1, a), ctx.h)
    end
    return s
end

"""Z3_s(N) = normalize(Z3(N,1) + Z3(N,2) + Z3(N,3)) (src/hilbert.jl:849)."""
gpu_Z3_s(N::Integer; prec::Symbol=:c128, ctx::GPUContext=default_context()) =
    _superpose(N, [_basis_index(_z3_bits(N, j)) for j in 1:3], prec, ctx)

"""neel_state_s(N) = (neel_state01(N) + neel_state10(N)) / sqrt(2) (src/hilbert.jl:854)."""
gpu_neel_state_s(N::Integer; prec::Symbol=:c128, ctx::GPUContext=default_context()) =
    _superpose(N, [_basis_index([isodd(i) ? 0 : 1 for i in 1:N]), _basis_index([isodd(i) ? 1 : 0 for i in 1:N])],
               prec, ctx)

# H on every qubit, as one compiled plan
function _all_h!(s::GPUState)
    p = gpu_compile([Op("H", q) for q in 1:s.n], s.n; prec=_prec_symbol(s), ctx=s.ctx)
    return run!(p, s)
end

"""plus_state(N) (src/hilbert.jl:869) and minus_state(N) (:871-877): H on every
qubit of |0...0> and of |1...1>."""
gpu_plus_state(N::Integer; prec::Symbol=:c128, ctx::GPUContext=default_context()) =
    _all_h!(_alloc(GPUState, N, prec, 1, ctx))
gpu_minus_state(N::Integer; prec::Symbol=:c128, ctx::GPUContext=default_context()) =
    _all_h!(gpu_one_state(N; prec=prec, ctx=ctx))

"""random_state(N) = normalize(rand(ComplexF64, 2^N)) (src/hilbert.jl:882), drawn
on the device (bt_state_random: real and imaginary parts uniform on [0, 1))."""
function gpu_random_state(N::Integer; seed::Integer=rand(UInt64), prec::Symbol=:c128,
                          ctx::GPUContext=default_context())
    s = _alloc(GPUState, N, prec, 1, ctx)
    check(ccall((:bt_state_random, lib), Cint, (Ptr{Cvoid}, Int64, UInt64), s.h, 0, seed % UInt64), ctx.h)
    return s
end

# ------------------------------------------------------------------ low level
_i32(xs) = Int32[Int32(x) for x in xs]
_kraus_buffer(kraus) = reduce(vcat, [vec(Matrix{ComplexF64}(k)) for k in kraus])

"""op.expand(N)*state (or e_op*rho*e_op') for a dense matrix on `qubits`
(src/hilbert.jl:469-515, :639-666)."""
function apply_matrix!(s::GPUHandle, mat::AbstractMatrix, qubits, controls=Int[]; member::Integer=-1)
    q = _i32(qubits)
    c = isempty(controls) ? Int32[0] : _i32(controls)
    M = Matrix{ComplexF64}(mat)  # column-major, as the ABI expects
    check(ccall((:bt_apply_matrix, lib), Cint,
                (Ptr{Cvoid}, Cint, Ptr{Int32}, Ptr{ComplexF64}, Cint, Ptr{Int32}, Int64),
                s.h, length(q), q, M, length(controls), isempty(controls) ? C_NULL : pointer(c), member), s.ctx.h)
    return s
end

"""QuantumChannel.apply / OpQC.apply (src/struct.jl:31-76): a Monte-Carlo branch
per member on a state (the reference's rand() draw), the Kraus sum on rho."""
function apply_channel!(s::GPUHandle, kraus, qubit::Integer, target::Integer=-1)
    k = round(Int, log2(size(kraus[1], 1)))
    qubits = k == 3 ? [qubit, qubit + 1, qubit + 2] : (k == 2 ? [qubit, target] : [qubit])
    k == 2 && target < 0 && throw(ArgumentError("for 2-qubit quantum channel, you must select the target_qubit"))
    q = _i32(qubits)
    K = _kraus_buffer(kraus)
    if s isa GPUDensity
        check(ccall((:bt_apply_kraus, lib), Cint,
                    (Ptr{Cvoid}, Cint, Ptr{Int32}, Cint, Ptr{ComplexF64}, Cint, Ptr{Float64}, Ptr{Int32}, Ptr{Int32},
                     Ptr{Float64}),
                    s.h, k, q, length(kraus), K, BT_KRAUS_SUM, C_NULL, C_NULL, C_NULL, C_NULL), s.ctx.h)
        return s
    end
    u = rand(s.batch)
    br = Vector{Int32}(undef, s.batch)
    pr = Vector{Float64}(undef, s.batch * length(kraus))
    check(ccall((:bt_apply_kraus, lib), Cint,
                (Ptr{Cvoid}, Cint, Ptr{Int32}, Cint, Ptr{ComplexF64}, Cint, Ptr{Float64}, Ptr{Int32}, Ptr{Int32},
                 Ptr{Float64}),
                s.h, k, q, length(kraus), K, BT_KRAUS_TRAJ | BT_KRAUS_REF_ORDER, u, C_NULL, br, pr), s.ctx.h)
    return s
end

"""born_measure_Z(N, psi, q) (src/hilbert.jl:682-696) in place: returns (state,
outcome); outcome is a vector over members for a batched state.  On a density
matrix: sum_b P_b rho P_b (src/hilbert.jl:784-796).
born_measure_Z!(N, psi, q1, q2) (src/hilbert.jl:705-721): outcome in 1..4, the
reference's index into [P0 P0, P1 P0, P0 P1, P1 P1] on (q1, q2)."""
function born_measure_Z!(N::Int, s::GPUHandle, qubit::Int)
    u = rand(s.batch)
    out = Vector{Int32}(undef, s.batch)
    p0 = Vector{Float64}(undef, s.batch)
    check(ccall((:bt_measure_z, lib), Cint, (Ptr{Cvoid}, Cint, Ptr{Float64}, Ptr{Int32}, Ptr{Int32}, Ptr{Float64}),
                s.h, qubit, u, C_NULL, out, p0), s.ctx.h)
    return s, (s.batch == 1 ? Int(out[1]) : Int.(out))
end

function born_measure_Z!(N::Int, s::GPUState, qubit1::Int, qubit2::Int)
    u = rand(s.batch)
    out = Vector{Int32}(undef, s.batch)
    probs = Vector{Float64}(undef, 4 * s.batch)
    check(ccall((:bt_measure_z2, lib), Cint,
                (Ptr{Cvoid}, Cint, Cint, Ptr{Float64}, Ptr{Int32}, Ptr{Int32}, Ptr{Float64}),
                s.h, qubit1, qubit2, u, C_NULL, out, probs), s.ctx.h)
    return s, (s.batch == 1 ? Int(out[1]) : Int.(out))
end

"""born_measure_Z as the reference has it: a new state, the argument unchanged."""
born_measure_Z(N::Int, s::GPUHandle, qubit::Int) = born_measure_Z!(N, copy(s), qubit)
born_measure_Z(N::Int, s::GPUState, qubit1::Int, qubit2::Int) = born_measure_Z!(N, copy(s), qubit1, qubit2)

# _born_measure (src/hilbert.jl:669-679): rotate into the basis, measure Z, rotate back
# the basis rotation of a measurement op; MR draws its basis at every use
# (src/struct.jl:554-576)
_measurement_rotation(op) = Matrix{ComplexF64}(BlueTangle._measurement_mat(BlueTangle._resolve_measurement_name(op.name)))

function _born_measure!(s::GPUHandle, op::QuantumOps)
    rot = _measurement_rotation(op)
    z = rot == I  # MZ: no rotation
    z || apply_matrix!(s, rot, [op.qubit])
    s, ind = born_measure_Z!(s.n, s, op.qubit)
    z || apply_matrix!(s, rot', [op.qubit])
    return s, ind
end

# _reset_Z (src/hilbert.jl:752-759): measure Z, flip the members that read 1
function _reset_Z!(s::GPUState, qubit::Int)
    s, ind = born_measure_Z!(s.n, s, qubit)
    X = ComplexF64[0 1; 1 0]
    if s.batch == 1
        ind == 1 && apply_matrix!(s, X, [qubit])
    else
        for m in findall(==(1), ind)
            apply_matrix!(s, X, [qubit]; member=m - 1)
        end
    end
    return s, ind
end

_qubits_of(op) = op.q == 1 ? [op.qubit] : [op.qubit, op.target_qubit]
_controls_of(op) = op.control == -2 ? Int[] : [op.control]

"""apply_noise (src/hilbert.jl:322-364) in place."""
function apply_noise!(s::GPUHandle, op::QuantumOps, noise)
    (noise isa NoiseModel && hasproperty(op, :noisy) && op.noisy) || return s
    if op.q == 1
        ch = op.control == -2 ? noise.q1 : noise.q2
        ch isa QuantumChannel || return s
        return op.control == -2 ? apply_channel!(s, ch.kraus, op.qubit) : apply_channel!(s, ch.kraus, op.control, op.qubit)
    elseif op.q == 2 && noise.q2 isa QuantumChannel
        return apply_channel!(s, noise.q2.kraus, op.qubit, op.target_qubit)
    end
    return s
end
apply_noise(s::GPUHandle, op::QuantumOps, noise::NoiseModel) = apply_noise!(copy(s), op, noise)

# ------------------------------------------------------------------ apply
function _apply_gate!(s::GPUHandle, op::QuantumOps; pars=nothing)
    mat = op.type == "f" ? op.mat(pars...) : op.mat
    if op.q == 1
        return apply_matrix!(s, mat, [op.qubit], _controls_of(op))
    end
    return apply_matrix!(s, mat, [op.qubit, op.target_qubit], _controls_of(op))
end

function _apply_one!(s::GPUHandle, op::QuantumOps, noise, pars)
    mids = Int[]
    dm = s isa GPUDensity
    if op isa OpF
        throw(ArgumentError("OpF acts through a host function: apply it to Vector(state)"))
    elseif op isa OpQC
        if uppercase(op.name) in ("RES", "RESET") && !dm
            _reset_Z!(s, op.qubit)
        else
            apply_channel!(s, op.kraus, op.qubit, op.q == 2 ? op.target_qubit : -1)
        end
    elseif op.type == "🔬"
        dm && throw(op isa ifOp ? "error: fix this!" : "fix this:")
        s, ind = _born_measure!(s, op)
        if op isa ifOp
            for sub in (ind == 0 ? op.if01[1] : op.if01[2])
                _apply_one!(s, sub, noise, pars)
            end
        end
        push!(mids, ind)
    else
        _apply_gate!(s, op; pars=pars)
    end
    if noise isa NoiseModel && !(op isa ifOp)
        apply_noise!(s, op, noise)
    end
    return s, mids
end

"""apply! (state, op(s); noise, track_measurements, pars): the reference's
apply (src/hilbert.jl:469-557, :639-666) acting on the handle in place."""
function apply!(s::GPUHandle, ops::AbstractVector; noise::Union{NoiseModel,Bool}=false,
                track_measurements::Bool=false, pars=nothing)
    mids = Int[]
    for op in ops
        o = op isa Tuple ? Op(op...) : op
        s, m = _apply_one!(s, o, noise, pars)
        append!(mids, m)
    end
    return track_measurements ? (s, mids) : s
end
apply!(s::GPUHandle, op::QuantumOps; kw...) = apply!(s, [op]; kw...)
apply!(s::GPUHandle, op::Tuple; kw...) = apply!(s, [Op(op...)]; kw...)

"""apply (src/hilbert.jl:469-557): a new state; the argument is left as it was."""
apply(s::GPUHandle, op::Union{QuantumOps,Tuple,AbstractVector}; kw...) = apply!(copy(s), op; kw...)
apply(op::Union{QuantumOps,Tuple}, s::GPUHandle; kw...) = apply(s, op; kw...)
apply(ops::AbstractVector, s::GPUHandle; kw...) = apply(s, ops; kw...)

# ------------------------------------------------------------------ sampling and observables
"""sample(psi, shots) (src/ops.jl:46-62): basis indices 0..2^N-1 of one member."""
function sample(s::GPUState, shots::Integer; member::Integer=0)
    out = Vector{Int64}(undef, shots)
    u = rand(shots)
    check(ccall((:bt_sample, lib), Cint, (Ptr{Cvoid}, Int64, Int64, Ptr{Float64}, UInt64, Ptr{Int64}),
                s.h, member, shots, u, UInt64(0), out), s.ctx.h)
    return out
end

"""sample_exact (src/ops.jl:98-101, :129-132): indices with non-zero weight, weights."""
function sample_exact(s::GPUHandle; member::Integer=0)
    out = Vector{Float64}(undef, 1 << s.n)
    check(ccall((:bt_probabilities, lib), Cint, (Ptr{Cvoid}, Int64, Ptr{Float64}), s.h, member, out), s.ctx.h)
    nz = findall(!iszero, out)
    return nz .- 1, out[nz]
end

"""measure(state, number_of_experiment) (src/ops.jl:496-513): the reference's
Measurement from the GPU's exact weights (-1) or from `number_of_experiment`
samples, built by the reference's own helpers."""
function measure(s::GPUState, number_of_experiment::Int=-1; label="state to measurement")
    N = s.n
    rho_construct = BlueTangle.sa.spzeros(ComplexF64, 2^N, 2^N)
    if number_of_experiment == -1
        bitstr, avg_prob = sample_exact(s)
    else
        bitstr, avg_prob = BlueTangle.get_probs_from_sample(collect(Int, sample(s, number_of_experiment)), N)
    end
    fock = int2bin.(bitstr, N)
    expect = [BlueTangle._sample_to_expectation((fock, avg_prob), [i]) for i = 1:N]
    mag_moments_list = [mag_moments(N, bitstr, avg_prob, moment_order) for moment_order = 1:12]
    return Measurement(bitstr, avg_prob, expect, mag_moments_list, "0", number_of_experiment, label, N, rho_construct)
end

const _PAULI = (("I", ComplexF64[1 0; 0 1]), ("X", ComplexF64[0 1; 1 0]),
                ("Y", ComplexF64[0 -im; im 0]), ("Z", ComplexF64[1 0; 0 -1]))

# a product of one-qubit matrices expanded into Pauli strings: (coef, xmask, zmask)
function _pauli_terms(mats, qubits, n)
    terms = Tuple{ComplexF64,UInt64,UInt64}[(1.0 + 0im, UInt64(0), UInt64(0))]
    for (M, q) in zip(mats, qubits)
        b = UInt64(1) << (n - q)
        new = Tuple{ComplexF64,UInt64,UInt64}[]
        for (name, P) in _PAULI
            c = tr(P * M) / 2
            c == 0 && continue
            x = name in ("X", "Y") ? b : UInt64(0)
            z = name in ("Z", "Y") ? b : UInt64(0)
            for (tc, tx, tz) in terms
                push!(new, (tc * c, tx | x, tz | z))
            end
        end
        terms = new
    end
    return terms
end

function _expect_terms(s::GPUHandle, terms; member::Integer=0)
    isempty(terms) && return 0.0
    xs = UInt64[t[2] for t in terms]
    zs = UInt64[t[3] for t in terms]
    out = Vector{Float64}(undef, length(terms))
    check(ccall((:bt_expect_pauli, lib), Cint,
                (Ptr{Cvoid}, Cint, Ptr{UInt64}, Ptr{UInt64}, Ptr{Float64}, Int64, Ptr{Float64}),
                s.h, length(terms), xs, zs, C_NULL, member, out), s.ctx.h)
    # Hermitian strings have real expectations: Re(c <P>) = Re(c) <P>
    return sum(real(t[1]) * v for (t, v) in zip(terms, out))
end

"""expect(state, "Z") / expect(state, "X") / expect(state, op) (src/func.jl:91-101)."""
function expect(s::GPUHandle, what::String; member::Integer=0)
    n = s.n
    if uppercase(what) == "Z"
        out = Vector{Float64}(undef, n)
        check(ccall((:bt_expect_z_all, lib), Cint, (Ptr{Cvoid}, Int64, Ptr{Float64}), s.h, member, out), s.ctx.h)
        return out
    end
    M = gates(what)
    return [_expect_terms(s, _pauli_terms([M], [q], n); member=member) for q in 1:n]
end

function expect(s::GPUHandle, op::QuantumOps; member::Integer=0)
    if s isa GPUState && op.q <= 2 && op.type != "f"
        q = _i32(_qubits_of(op))
        ctrls = _controls_of(op)
        c = isempty(ctrls) ? Int32[0] : _i32(ctrls)
        M = Matrix{ComplexF64}(op.mat)
        out = Ref{Float64}(0.0)
        check(ccall((:bt_expect_matrix, lib), Cint,
                    (Ptr{Cvoid}, Cint, Ptr{Int32}, Ptr{ComplexF64}, Cint, Ptr{Int32}, Int64, Ref{Float64}),
                    s.h, length(q), q, M, length(ctrls), isempty(ctrls) ? C_NULL : pointer(c), member, out), s.ctx.h)
        return out[]
    end
    # density matrix: Re tr(rho E) through the Pauli expansion of E
    if op.q == 1 && op.control == -2
        return _expect_terms(s, _pauli_terms([op.mat], [op.qubit], s.n); member=member)
    end
    throw(ArgumentError("expect(rho, op) supports uncontrolled one-qubit ops; use correlation for strings"))
end

"""correlation(state, "Z,Z", [i, j]) (src/func.jl:139-147)."""
function correlation(s::GPUHandle, list_of_operators::String, qubits_applied::Vector; member::Integer=0)
    names = strip.(split(list_of_operators, ","))
    length(names) == length(qubits_applied) || throw("qubit number does not match with operators")
    mats = [gates(String(x)) for x in names]
    return _expect_terms(s, _pauli_terms(mats, qubits_applied, s.n); member=member)
end

"""fidelity(psi, phi) = |<psi|phi>|^2 (src/tensor.jl:219) and, for density
matrices, tr(sqrt(sqrt(rho) sigma sqrt(rho)))^2 (src/tensor.jl:222-229)."""
function fidelity(a::GPUHandle, b::GPUHandle; amember::Integer=0, bmember::Integer=0)
    out = Ref{Float64}(0.0)
    sym = (a isa GPUDensity || b isa GPUDensity) ? :bt_fidelity_dm : :bt_fidelity
    if sym === :bt_fidelity_dm
        check(ccall((:bt_fidelity_dm, lib), Cint, (Ptr{Cvoid}, Int64, Ptr{Cvoid}, Int64, Ref{Float64}),
                    a.h, amember, b.h, bmember, out), a.ctx.h)
    else
        check(ccall((:bt_fidelity, lib), Cint, (Ptr{Cvoid}, Int64, Ptr{Cvoid}, Int64, Ref{Float64}),
                    a.h, amember, b.h, bmember, out), a.ctx.h)
    end
    return out[]
end

# ------------------------------------------------------------------ compiled circuits
"""A compiled circuit (bt_plan): gates (and, for density matrices, Kraus sums)
fused into tile passes; running it equals applying the ops one by one."""
mutable struct GPUPlan
    h::Ptr{Cvoid}
    ctx::GPUContext
    n::Int
end

function _plan_check(p::GPUPlan, rc::Cint)
    return check(rc, p.ctx.h)
end

function gpu_compile(ops::AbstractVector, N::Integer; density::Bool=false, prec::Symbol=:c128,
                     tiered::Bool=false, tensor_cores::Bool=false, ctx::GPUContext=default_context())
    r = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:bt_plan_create, lib), Cint, (Ptr{Cvoid}, Cint, Cint, Cint, Ptr{Ptr{Cvoid}}),
                ctx.h, N, density ? BT_REPR_DM : BT_REPR_SV, PRECISIONS[prec], r), ctx.h)
    p = finalizer(GPUPlan(r[], ctx, Int(N))) do x
        x.h != C_NULL && ccall((:bt_plan_free, lib), Cint, (Ptr{Cvoid},), x.h)
        x.h = C_NULL
    end
    for op in ops
        if op isa OpQC
            density || throw(ArgumentError("channels in a state-vector plan need trajectories; apply them with apply"))
            op.q <= 2 || throw(ArgumentError("3-qubit OpQC has no density-matrix method in the reference"))
            q = _i32(_qubits_of(op))
            K = _kraus_buffer(op.kraus)
            _plan_check(p, ccall((:bt_plan_add_kraus_sum, lib), Cint,
                                 (Ptr{Cvoid}, Cint, Ptr{Int32}, Cint, Ptr{ComplexF64}),
                                 p.h, length(q), q, length(op.kraus), K))
        elseif op.type == "🔬"
            throw(ArgumentError("measurements end a plan"))
        else
            q = _i32(_qubits_of(op))
            ctrls = _controls_of(op)
            c = isempty(ctrls) ? Int32[0] : _i32(ctrls)
            # a parametrised op enters with zero angles: set_matrices! gives the real ones
            M = Matrix{ComplexF64}(op.type == "f" ? op.mat(zeros(BlueTangle._find_argument_number(op.mat))...) : op.mat)
            _plan_check(p, ccall((:bt_plan_add_matrix, lib), Cint,
                                 (Ptr{Cvoid}, Cint, Ptr{Int32}, Ptr{ComplexF64}, Cint, Ptr{Int32}),
                                 p.h, length(q), q, M, length(ctrls), isempty(ctrls) ? C_NULL : pointer(c)))
        end
    end
    mode = tensor_cores ? 3 : (tiered ? 2 : 0)
    _plan_check(p, ccall((:bt_plan_compile, lib), Cint, (Ptr{Cvoid}, Cint), p.h, mode))
    return p
end

"""gpu_compile with the parametrised (type "f") ops marked variable: their
matrices are encoded in entry-independent forms, so set_matrices! never
recompiles."""
function gpu_compile_variational(ops::AbstractVector, N::Integer; kw...)
    p = gpu_compile(ops, N; kw...)
    var = Int64[i - 1 for (i, op) in enumerate(ops) if !(op isa OpQC) && op.type == "f"]
    _plan_check(p, ccall((:bt_plan_set_variable, lib), Cint, (Ptr{Cvoid}, Cint, Ptr{Int64}), p.h, length(var), var))
    _plan_check(p, ccall((:bt_plan_compile, lib), Cint, (Ptr{Cvoid}, Cint), p.h, 0))
    return p
end

"""New matrices for gates already added (add_index counts the ops from 0)."""
function set_matrices!(p::GPUPlan, add_index::Vector{Int64}, mats::Vector{<:AbstractMatrix})
    buf = reduce(vcat, [vec(Matrix{ComplexF64}(m)) for m in mats])
    _plan_check(p, ccall((:bt_plan_set_matrices, lib), Cint, (Ptr{Cvoid}, Cint, Ptr{Int64}, Ptr{ComplexF64}),
                         p.h, length(add_index), add_index, buf))
    return p
end

"""Real flops and HBM bytes per amplitude of one run."""
function plan_cost(p::GPUPlan)
    f, b = Ref{Float64}(0.0), Ref{Float64}(0.0)
    _plan_check(p, ccall((:bt_plan_cost, lib), Cint, (Ptr{Cvoid}, Ref{Float64}, Ref{Float64}), p.h, f, b))
    return f[], b[]
end

function run!(p::GPUPlan, s::GPUHandle; member::Integer=-1)
    check(ccall((:bt_plan_run, lib), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Int64), p.h, s.h, member), s.ctx.h)
    return s
end

"""Every member of s through the plan, member m with mats[m] (one matrix per add
index in idx) for those gates: one launch per pass for the whole batch."""
function run_members!(p::GPUPlan, s::GPUState, idx::Vector{Int64}, mats::Vector{<:Vector{<:AbstractMatrix}})
    length(mats) == s.batch || throw(ArgumentError("one list of matrices per member"))
    buf = reduce(vcat, [vec(Matrix{ComplexF64}(m)) for mm in mats for m in mm])
    check(ccall((:bt_plan_run_members, lib), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ptr{Int64}, Ptr{ComplexF64}),
                p.h, s.h, length(idx), idx, buf), s.ctx.h)
    return s
end

# ------------------------------------------------------------------ variational circuits
"""gpu_variational_apply(pars, opt; noise_override): variational_apply(pars, opt)
(src/vqa.jl:420-456) on the GPU: opt.init uploaded, every op applied with its
slice of pars, the NoiseModel (opt.noise, or noise_override) after each op."""
function gpu_variational_apply(pars::AbstractVector, opt::AnsatzOptions; noise_override::Union{Bool,NoiseModel}=false,
                               prec::Symbol=:c128, ctx::GPUContext=default_context())
    s = _initial_members!(_alloc(GPUState, opt.N, prec, 1, ctx), opt.init)
    noise = noise_override isa NoiseModel ? noise_override : opt.noise
    c = 1
    for (op, fn) in zip(opt.ops, opt.args)
        fn > 0 ? apply!(s, op; pars=pars[c:c+fn-1]) : apply!(s, op)
        c += fn
        noise isa NoiseModel && !(op isa OpQC) && apply_noise!(s, op, noise)
    end
    return s
end

# every member set to the ansatz's initial state (|0...0> when it is one)
function _initial_members!(s::GPUState, init)
    flat = Vector{ComplexF64}(init)
    length(flat) == (1 << s.n) || throw(ArgumentError("the initial state has $(length(flat)) entries, not 2^$(s.n)"))
    if flat[1] == 1 && count(!iszero, flat) == 1
        return set_zero!(s)
    end
    for m in 0:s.batch-1
        _upload!(s, flat, m)
    end
    return s
end

# Hamiltonian terms [(coef, "Z,Z", [i, j]), ...] as Pauli strings (coef, xmask, zmask)
function _hamiltonian_terms(terms, n)
    out = Tuple{ComplexF64,UInt64,UInt64}[]
    for (c, names, qubits) in terms
        mats = [gates(String(strip(x))) for x in split(names, ",")]
        length(mats) == length(qubits) || throw("qubit number does not match with operators")
        append!(out, [(c * tc, x, z) for (tc, x, z) in _pauli_terms(mats, qubits, n)])
    end
    return out
end

# sum_t Re(c_t) <P_t> of every member (bt_expect_pauli over the batch, FP64 sums)
function _expect_members(s::GPUState, terms)
    isempty(terms) && return zeros(s.batch)
    xs = UInt64[t[2] for t in terms]
    zs = UInt64[t[3] for t in terms]
    out = Vector{Float64}(undef, length(terms) * s.batch)
    check(ccall((:bt_expect_pauli, lib), Cint,
                (Ptr{Cvoid}, Cint, Ptr{UInt64}, Ptr{UInt64}, Ptr{Float64}, Int64, Ptr{Float64}),
                s.h, length(terms), xs, zs, C_NULL, -1, out), s.ctx.h)
    v = reshape(out, length(terms), s.batch)  # member-major
    return [sum(real(t[1]) * v[i, m] for (i, t) in enumerate(terms)) for m in 1:s.batch]
end

# matrices of the parametrised ops at p, by op index
function _bound_mats(opt::AnsatzOptions, p::AbstractVector)
    sum(opt.args) == length(p) || throw(ArgumentError("the ansatz takes $(sum(opt.args)) parameters, $(length(p)) given"))
    mats = Dict{Int,Matrix{ComplexF64}}()
    c = 1
    for (j, (op, fn)) in enumerate(zip(opt.ops, opt.args))
        if fn > 0
            mats[j] = Matrix{ComplexF64}(op.mat(p[c:c+fn-1]...))
            c += fn
        end
    end
    return mats
end

const _MEMBER_BUDGET = 16 << 30  # HBM for the members of one batched run

# the loss of every evaluation (a Dict of the parametrised ops' matrices each):
# noiseless ansatze as members of one compiled plan, each member with its own
# matrices (bt_plan_run_members), in chunks that fit _MEMBER_BUDGET; noisy ones
# one trajectory per evaluation, as the reference evaluates them
function _losses(opt::AnsatzOptions, evals::Vector{Dict{Int,Matrix{ComplexF64}}}, params, terms, prec, ctx)
    N = opt.N
    hterms = terms === nothing ? nothing : _hamiltonian_terms(terms, N)
    lossof(s, m) = hterms === nothing ? opt.loss(BlueTangle.sa.sparse(Vector(s; member=m))) :
                   _expect_terms(s, hterms; member=m)
    if opt.noise isa NoiseModel || any(op -> op isa OpQC || op.type == "🔬", opt.ops)
        return [lossof(gpu_variational_apply(p, opt; prec=prec, ctx=ctx), 0) for p in params]
    end
    plan = gpu_compile_variational(opt.ops, N; prec=prec, ctx=ctx)
    var = sort(collect(keys(evals[1])))
    idx = Int64[j - 1 for j in var]
    bytes = (1 << N) * (prec == :c64 ? 8 : 16)
    chunk = max(1, min(length(evals), _MEMBER_BUDGET ÷ bytes))
    vals = Vector{Float64}(undef, length(evals))
    for e0 in 1:chunk:length(evals)
        es = e0:min(length(evals), e0 + chunk - 1)
        s = _initial_members!(_alloc(GPUState, N, prec, length(es), ctx), opt.init)
        run_members!(plan, s, idx, [[evals[e][j] for j in var] for e in es])
        vals[es] = hterms === nothing ? [lossof(s, m) for m in 0:length(es)-1] : _expect_members(s, hterms)
    end
    return vals
end

"""gpu_loss_and_grad_paramshift(p, opt; terms): loss_and_grad_paramshift(p, opt)
(src/vqa.jl:590-611) on the GPU: the loss at p and, for every parameter i,
g_i = (l(p + pi/2 e_i) - l(p - pi/2 e_i)) / 2, all 2P + 1 evaluations as one
batch.  The loss is sum_t c_t <P_t> of `terms` [(coef, "Z,Z", [i, j]), ...] on
the device, or, without terms, the ansatz's own opt.loss on each evaluated state
(downloaded)."""
function gpu_loss_and_grad_paramshift(p::Vector{Float64}, opt::AnsatzOptions; terms=nothing, prec::Symbol=:c128,
                                      ctx::GPUContext=default_context())
    SHIFT = pi / 2
    base = _bound_mats(opt, p)
    params = [copy(p)]
    evals = [base]
    owner = Int[]  # op of each parameter
    for (j, fn) in enumerate(opt.args), _ in 1:fn
        push!(owner, j)
    end
    for i in eachindex(p), sh in (SHIFT, -SHIFT)
        q = copy(p)
        q[i] += sh
        push!(params, q)
        m = copy(base)
        m[owner[i]] = _bound_mats(opt, q)[owner[i]]
        push!(evals, m)
    end
    vals = _losses(opt, evals, params, terms, prec, ctx)
    g = [0.5 * (vals[2i] - vals[2i+1]) for i in eachindex(p)]
    return (vals[1], g)
end

"""gpu_loss(p, opt; terms): the loss of the ansatz at p (_loss, src/vqa.jl:588)."""
gpu_loss(p::Vector{Float64}, opt::AnsatzOptions; terms=nothing, prec::Symbol=:c128, ctx::GPUContext=default_context()) =
    _losses(opt, [_bound_mats(opt, p)], [p], terms, prec, ctx)[1]

# ------------------------------------------------------------------ noisy shots (programs)
"""A noisy circuit run on every member of a batch (bt_program): the per-shot loop
of measure(circuit, shots) (src/ops.jl:599-646) as one launch sequence."""
mutable struct GPUProgram
    h::Ptr{Cvoid}
    ctx::GPUContext
    n::Int
    batch::Int
    nrec::Int
end

_program_check(p::GPUProgram, rc::Cint) = check(rc, p.ctx.h)

# |0><0| (x) I + |1><1| (x) U on (control, target), the control the matrix's MSB
function _ctrl_matrix(mat::AbstractMatrix)
    d = size(mat, 1)
    M = Matrix{ComplexF64}(I, 2d, 2d)
    M[d+1:end, d+1:end] = mat
    return M
end

# Kraus operators that are multiples of unitaries: the branch is drawn from |c_i|^2
_unitary_mix(kraus) = all(K -> (P = K' * K; isapprox(P, P[1, 1] * I; atol=1e-12)), kraus)

function _program_gate!(p::GPUProgram, mat::AbstractMatrix, qubits)
    q = _i32(qubits)
    M = Matrix{ComplexF64}(mat)
    _program_check(p, ccall((:bt_program_add_gate, lib), Cint, (Ptr{Cvoid}, Cint, Ptr{Int32}, Ptr{ComplexF64}, Cint),
                            p.h, length(q), q, M, 0))
end

function _program_channel!(p::GPUProgram, kraus, qubits)
    q = _i32(qubits)
    K = _kraus_buffer(kraus)
    flags = BT_KRAUS_TRAJ | BT_KRAUS_REF_ORDER | (_unitary_mix(kraus) ? BT_KRAUS_UNITARY_MIX : Cint(0))
    _program_check(p, ccall((:bt_program_add_channel, lib), Cint,
                            (Ptr{Cvoid}, Cint, Ptr{Int32}, Cint, Ptr{ComplexF64}, Cint, Ptr{Int32}),
                            p.h, length(q), q, length(kraus), K, flags, C_NULL))
end

function _program_measure!(p::GPUProgram, op)
    rot = _measurement_rotation(op)
    z = rot == I  # MZ: no rotation
    z || _program_gate!(p, rot, [op.qubit])
    _program_check(p, ccall((:bt_program_add_measure, lib), Cint, (Ptr{Cvoid}, Cint, Ptr{Int32}),
                            p.h, op.qubit, C_NULL))
    p.nrec += 1
    z || _program_gate!(p, rot', [op.qubit])
end

# the ops of one shot with ZNE repetitions (_expanded_ops_for_shot, src/ops.jl:555-573)
function _expanded_ops(ops, id::Integer)
    out = QuantumOps[]
    for op in ops
        if id > 0 && op.q == 2 && uppercase(op.name) in ("CNOT", "CX")
            for _ in 1:(2id+1)
                push!(out, op)
            end
        else
            push!(out, op)
        end
    end
    return out
end

"""gpu_shots(ops, N, shots; noise, id, seed): every shot of a noisy circuit as one
member of a batch, run as one program (one CTA per shot in shared memory up to 14
qubits complex64 / 13 complex128, the grouped executor beyond).  Controlled
one-qubit gates enter as the 4x4 |0><0| (x) I + |1><1| (x) U on (control,
target); a NoiseModel adds its channels after every noisy op (src/hilbert.jl:
322-340); OpQC("RES") is the reference's reset channel {|0><0|, |0><1|}, whose
branch is the reset's measured outcome.  Returns (states, records) with
records[:, shot] the mid-circuit outcomes of that shot."""
function gpu_shots(ops::AbstractVector, N::Integer, shots::Integer; noise::Union{NoiseModel,Bool}=false,
                   id::Integer=0, seed::Integer=rand(UInt64), prec::Symbol=:c64,
                   ctx::GPUContext=default_context())
    p = _shot_program(_expanded_ops(ops, id), N, shots, noise, prec, ctx)
    return _run_program(p, N, shots, prec, seed, ctx)
end

# the program of a circuit's ops (and the NoiseModel's channels after every noisy
# op), one member per shot
function _shot_program(ops, N, shots, noise, prec, ctx)
    r = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:bt_program_create, lib), Cint, (Ptr{Cvoid}, Cint, Cint, Cint, Ptr{Ptr{Cvoid}}),
                ctx.h, N, PRECISIONS[prec], shots, r), ctx.h)
    p = finalizer(GPUProgram(r[], ctx, Int(N), Int(shots), 0)) do x
        x.h != C_NULL && ccall((:bt_program_free, lib), Cint, (Ptr{Cvoid},), x.h)
        x.h = C_NULL
    end
    for op in ops
        if op isa ifOp
            throw(ArgumentError("classically controlled ops follow each shot's outcomes: apply! them per shot"))
        elseif op isa OpQC
            _program_channel!(p, op.kraus, op.q == 1 ? [op.qubit] :
                                           (op.q == 2 ? [op.qubit, op.target_qubit] : [op.qubit, op.qubit + 1, op.qubit + 2]))
            continue
        elseif op.type == "🔬"
            _program_measure!(p, op)
            continue
        elseif op.type == "f"
            throw(ArgumentError("parametrised op $(op.name): evaluate its matrix at the pars first"))
        elseif op.control != -2
            _program_gate!(p, _ctrl_matrix(op.mat), [op.control, op.qubit])
        else
            _program_gate!(p, op.mat, _qubits_of(op))
        end
        if noise isa NoiseModel && hasproperty(op, :noisy) && op.noisy
            if op.q == 1
                ch = op.control == -2 ? noise.q1 : noise.q2
                ch isa QuantumChannel && _program_channel!(p, ch.kraus, op.control == -2 ? [op.qubit] : [op.control, op.qubit])
            elseif noise.q2 isa QuantumChannel
                _program_channel!(p, noise.q2.kraus, [op.qubit, op.target_qubit])
            end
        end
    end
    return p
end

function _run_program(p::GPUProgram, N, shots, prec, seed, ctx)
    s = _alloc(GPUState, N, prec, shots, ctx)
    recs = Matrix{Int32}(undef, max(p.nrec, 1), shots)  # member-major: a column per shot
    check(ccall((:bt_program_run, lib), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Float64}, UInt64, Ptr{Int32}),
                p.h, s.h, C_NULL, seed % UInt64, recs), ctx.h)
    return s, recs[1:p.nrec, :]
end

"""One basis-state sample per shot of gpu_shots' batch (bt_sample_members): the
sample of the noisy measure(circuit, shots); measure(samples, N)
(src/ops.jl:516) turns it into the reference's Measurement."""
function gpu_shot_samples(ops::AbstractVector, N::Integer, shots::Integer; seed::Integer=rand(UInt64), kw...)
    s, _ = gpu_shots(ops, N, shots; seed=seed, kw...)
    return _member_samples(s, seed)
end

function _member_samples(s::GPUState, seed)
    out = Vector{Int64}(undef, s.batch)
    check(ccall((:bt_sample_members, lib), Cint, (Ptr{Cvoid}, Ptr{Float64}, UInt64, Ptr{Int64}),
                s.h, C_NULL, (seed + 1) % UInt64, out), s.ctx.h)
    return out
end

# ------------------------------------------------------------------ circuit drivers
"""gpu_to_state(circuit, id): to_state(circuit, id) (src/ops.jl:790-795) on the GPU:
the shot's ops (_expanded_ops_for_shot: twirl frames, ZNE repetitions) applied to
|0...0> with the circuit's noise."""
function gpu_to_state(circuit::Circuit, id::Int=0; prec::Symbol=:c128, ctx::GPUContext=default_context())
    s = _alloc(GPUState, circuit.stats.N, prec, 1, ctx)
    return apply!(s, BlueTangle._expanded_ops_for_shot(circuit, id); noise=circuit.options.noise)
end

"""gpu_to_rho(circuit; id): to_rho(circuit; id) (src/ops.jl:806-844) on the GPU,
with that function's own expansion: 2id+1 repetitions of the ops named exactly
CNOT or CX, apply_twirl around every two-qubit op when twirl is on, and the
NoiseModel's channels as Kraus sums."""
function gpu_to_rho(circuit::Circuit; id::Int=0, prec::Symbol=:c128, ctx::GPUContext=default_context())
    rho = _alloc(GPUDensity, circuit.stats.N, prec, 1, ctx)
    nm = circuit.options.noise
    tw = circuit.options.twirl
    for op in vcat(circuit.layers...)
        if op.q == 2 && (op.name == "CNOT" || op.name == "CX") && id > 0
            for _ in 1:(2id+1)
                apply!(rho, tw ? BlueTangle.apply_twirl(op) : [op]; noise=nm)
            end
        elseif op.q == 2 && tw
            apply!(rho, BlueTangle.apply_twirl(op); noise=nm)
        else
            apply!(rho, op; noise=nm)
        end
    end
    return rho
end

"""gpu_run(circuit, shots; id): run(circuit, shots; backend=:statevector, id)
(src/ops.jl:659-692) on the GPU: every shot's mid-circuit measurement outcomes.
Shots that run the same ops are the members of one program (gpu_shots); with
twirl frames or ifOps, which differ between shots, each shot runs with apply!."""
function gpu_run(circuit::Circuit, number_of_experiment::Int=1; id::Int=0, prec::Symbol=:c128,
                 seed::Integer=rand(UInt64), ctx::GPUContext=default_context())
    number_of_experiment > 0 || throw(ArgumentError("`number_of_experiment` must be positive."))
    N = circuit.stats.N
    nm = circuit.options.noise
    ops = BlueTangle._expanded_ops_for_shot(circuit, id)
    if circuit.options.twirl || any(op -> op isa ifOp || op isa OpF, ops)
        out = Vector{Vector{Int}}(undef, number_of_experiment)
        s = _alloc(GPUState, N, prec, 1, ctx)
        for shot in 1:number_of_experiment
            set_zero!(s)
            _, out[shot] = apply!(s, shot == 1 ? ops : BlueTangle._expanded_ops_for_shot(circuit, id);
                                  noise=nm, track_measurements=true)
        end
        return out
    end
    p = _shot_program(ops, N, number_of_experiment, nm, prec, ctx)
    _, recs = _run_program(p, N, number_of_experiment, prec, seed, ctx)
    return [Int.(recs[:, m]) for m in 1:number_of_experiment]
end

"""gpu_run(ops, shots; options, layout, id) and gpu_run(qasm_or_path, shots; ...):
the reference's run methods for op lists and OpenQASM (src/ops.jl:713-727): the
ops compiled by the reference's compile (from_qasm first for QASM), then gpu_run
of the circuit."""
gpu_run(ops::Vector{<:QuantumOps}, number_of_experiment::Int=1; options::Options=Options(),
        layout::Union{Layout,Int}=-1, id::Int=0, kw...) =
    gpu_run(compile(ops, options; layout=layout), number_of_experiment; id=id, kw...)
gpu_run(qasm_or_path::AbstractString, number_of_experiment::Int=1; options::Options=Options(),
        layout::Union{Layout,Int}=-1, id::Int=0, is_file::Union{Nothing,Bool}=nothing, kw...) =
    gpu_run(from_qasm(BlueTangle._qasm_to_source(qasm_or_path; is_file=is_file)), number_of_experiment;
            options=options, layout=layout, id=id, kw...)

# ------------------------------------------------------------------ measure(circuit, shots, id)
# the rotation of _final_measurement (src/ops.jl:856-914) for a basis; "R" draws one
# of H, HSP, I per qubit at every use
_basis_rotation(basis::String) = basis == "Z" ? ComplexF64[1 0; 0 1] :
                                 basis == "X" ? Matrix{ComplexF64}(BlueTangle.gate.H) :
                                 basis == "Y" ? Matrix{ComplexF64}(BlueTangle.gate.HSP) :
                                 basis == "R" ? Matrix{ComplexF64}([BlueTangle.gate.H, BlueTangle.gate.HSP, BlueTangle.gate.I][rand(1:3)]) :
                                 throw("measurement_basis error!")

# _final_measurement (src/ops.jl:856-914) in place: per qubit the basis rotation,
# then the readout channel's branch
function _final_measurement!(s::GPUState, o)
    for q in 1:s.n
        U = _basis_rotation(o.measurement_basis)
        U == I || apply_matrix!(s, U, [q])
        o.readout_noise isa QuantumChannel && apply_channel!(s, o.readout_noise.kraus, q)
    end
    return s
end

# sum_m w |psi_m><psi_m| of every member into a new density matrix (bt_rho_accumulate)
function _density_of(s::GPUState, w::Float64)
    rho = _alloc(GPUDensity, s.n, :c128, 1, s.ctx)
    check(ccall((:bt_state_clear, lib), Cint, (Ptr{Cvoid}, Int64), rho.h, -1), s.ctx.h)
    check(ccall((:bt_rho_accumulate, lib), Cint, (Ptr{Cvoid}, Int64, Ptr{Cvoid}, Float64), rho.h, 0, s.h, w), s.ctx.h)
    return rho
end

"""gpu_measure(circuit, number_of_experiment, id): measure(circuit,
number_of_experiment, id) (src/ops.jl:599-646) on the GPU, returning the
reference's Measurement.  A noiseless circuit runs once and is sampled; otherwise
every shot is one member of a batch: as one program (gpu_shots, with the final
rotation and readout channel appended) where every shot runs the same ops, shot by
shot (the reference's re-simulation, with apply!) where twirl frames, a random
basis or classically controlled ops differ between shots.  The density matrix, when
the options ask for it, is accumulated on the GPU and returned in the record as the
reference's sparse matrix; mitigation uses the reference's own inverse."""
function gpu_measure(circuit::Circuit, number_of_experiment::Int, id::Int=0; prec::Symbol=:c128,
                     seed::Integer=rand(UInt64), ctx::GPUContext=default_context())
    number_of_experiment > 0 || throw("`number_of_experiment` must be positive.")
    N = circuit.stats.N
    o = circuit.options
    rho = nothing
    noiseless = o.noise == false && circuit.stats.mid_measurement_count == 0 && !(o.readout_noise isa QuantumChannel)
    if noiseless
        s = _alloc(GPUState, N, prec, 1, ctx)
        apply!(s, BlueTangle._expanded_ops_for_shot(circuit, 0))
        _final_measurement!(s, o)
        samples = collect(Int, sample(s, number_of_experiment))
        o.density_matrix && (rho = _density_of(s, 1.0))
    else
        ops = BlueTangle._expanded_ops_for_shot(circuit, id)
        per_shot = o.twirl || o.measurement_basis == "R" || any(op -> op isa ifOp, ops)
        if per_shot
            s = _alloc(GPUState, N, prec, number_of_experiment, ctx)
            one = _alloc(GPUState, N, prec, 1, ctx)
            for m in 0:number_of_experiment-1
                set_zero!(one)
                apply!(one, m == 0 ? ops : BlueTangle._expanded_ops_for_shot(circuit, id); noise=o.noise)
                _final_measurement!(one, o)
                copy_from!(s, one; dst_member=m, src_member=0)
            end
        else
            p = _shot_program(ops, N, number_of_experiment, o.noise, prec, ctx)
            U = _basis_rotation(o.measurement_basis)
            for q in 1:N
                U == I || _program_gate!(p, U, [q])
                o.readout_noise isa QuantumChannel && _program_channel!(p, o.readout_noise.kraus, [q])
            end
            s, _ = _run_program(p, N, number_of_experiment, prec, seed, ctx)
        end
        samples = collect(Int, _member_samples(s, seed))
        o.density_matrix && (rho = _density_of(s, 1.0 / number_of_experiment))
    end
    bitstr, avg_prob = BlueTangle.get_probs_from_sample(samples, N)
    if o.measurement_mitigate && o.readout_noise isa QuantumChannel
        avg_prob = normalize(abs.(BlueTangle._measurement_mitigate_inv_matrix(N, o.readout_noise) * avg_prob), 1)
    end
    fock = int2bin.(bitstr, N)
    expect = [BlueTangle._sample_to_expectation((fock, avg_prob), [i]) for i = 1:N]
    mag_moments_list = [mag_moments(N, bitstr, avg_prob, moment_order) for moment_order = 1:12]
    rho_construct = rho === nothing ? BlueTangle.sa.spzeros(ComplexF64, 2^N, 2^N) : BlueTangle.sa.sparse(Matrix(rho))
    return Measurement(bitstr, avg_prob, expect, mag_moments_list, o.measurement_basis, number_of_experiment,
                       o.circuit_name, N, rho_construct)
end

# ------------------------------------------------------------------ classical shadows
"""gpu_shadow(circuit, number_of_experiment): shadow(circuit, number_of_experiment)
(src/ops.jl:145-185) on the GPU.  Every snapshot is one member of a batch: the
circuit (to_state), a random basis per qubit (H, HSP or I, the reference's m_list)
and a Z measurement of every qubit, whose joint outcome follows the rotated state's
Born distribution as the reference's one sample does; the snapshots
(x)_q (3 U'|b><b|U - I) / shots are summed into a density matrix on the device
(bt_shadow_accumulate, n <= 14).  Twirled circuits and ifOps, which differ between
shots, run shot by shot."""
function gpu_shadow(circuit::Circuit, number_of_experiment::Int; prec::Symbol=:c128,
                    seed::Integer=rand(UInt64), ctx::GPUContext=default_context())
    number_of_experiment > 0 || throw(ArgumentError("`number_of_experiment` must be positive."))
    N = circuit.stats.N
    shots = number_of_experiment
    m_list = [Matrix{ComplexF64}(BlueTangle.gate.H), Matrix{ComplexF64}(BlueTangle.gate.HSP), ComplexF64[1 0; 0 1]]
    bases = rand(1:3, shots, N)
    outcomes = Matrix{Int}(undef, shots, N)
    ops = BlueTangle._expanded_ops_for_shot(circuit, 0)
    if circuit.options.twirl || any(op -> op isa ifOp || op isa OpF, ops)
        for m in 1:shots
            s = gpu_to_state(circuit; prec=prec, ctx=ctx)
            for q in 1:N
                apply_matrix!(s, m_list[bases[m, q]], [q])
            end
            outcomes[m, :] = int2bin(Int(sample(s, 1)[1]), N)
        end
    else
        p = _shot_program(ops, N, shots, circuit.options.noise, prec, ctx)
        for q in 1:N
            buf = reduce(vcat, [vec(m_list[bases[m, q]]) for m in 1:shots])
            _program_check(p, ccall((:bt_program_add_gate, lib), Cint,
                                    (Ptr{Cvoid}, Cint, Ptr{Int32}, Ptr{ComplexF64}, Cint), p.h, 1, Int32[q], buf, 1))
        end
        for q in 1:N
            _program_check(p, ccall((:bt_program_add_measure, lib), Cint, (Ptr{Cvoid}, Cint, Ptr{Int32}),
                                    p.h, q, C_NULL))
            p.nrec += 1
        end
        _, recs = _run_program(p, N, shots, prec, seed, ctx)
        outcomes .= permutedims(recs[end-N+1:end, :])
        any(<(0), outcomes) && throw("a snapshot measurement failed")
    end
    # codes[m*N + q] (0-based) = 2*basis + outcome; the six factors row-major
    codes = UInt8[2 * (bases[m, q] - 1) + outcomes[m, q] for q in 1:N, m in 1:shots]
    tables = Float64[]
    for U in m_list, o in 0:1
        v = o == 0 ? ComplexF64[1, 0] : ComplexF64[0, 1]
        T = 3 * (U' * v * v' * U) - I
        for r in 1:2, c in 1:2
            push!(tables, real(T[r, c]), imag(T[r, c]))
        end
    end
    rho = _alloc(GPUDensity, N, prec, 1, ctx)
    check(ccall((:bt_shadow_accumulate, lib), Cint, (Ptr{Cvoid}, Int64, Ptr{UInt8}, Ptr{Float64}),
                rho.h, shots, vec(codes), tables), ctx.h)
    t = Ref{Float64}(0.0)
    check(ccall((:bt_norm2, lib), Cint, (Ptr{Cvoid}, Int64, Ref{Float64}), rho.h, 0, t), ctx.h)
    isapprox(t[], 1) || throw("la.tr(rho)!≈1")
    return rho
end

# ------------------------------------------------------------------ serving
"""The serving engine (bt_serve): client states resident, requests of different
clients run concurrently on lanes, a client's requests in order."""
mutable struct GPUServer
    h::Ptr{Cvoid}
end
function GPUServer(; device::Integer=0, lanes::Integer=8, seed::Integer=1234, hbm_budget::Integer=0)
    r = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:bt_serve_create, lib), Cint, (Cint, Cint, UInt64, UInt64, Ptr{Ptr{Cvoid}}),
                device, lanes, seed % UInt64, hbm_budget % UInt64, r), C_NULL)
    return finalizer(GPUServer(r[])) do x
        x.h != C_NULL && ccall((:bt_serve_destroy, lib), Cint, (Ptr{Cvoid},), x.h)
        x.h = C_NULL
    end
end

"""A client: a compiled plan and H as Pauli masks with coefficients."""
function add_client(s::GPUServer, p::GPUPlan, xmask::Vector{UInt64}, zmask::Vector{UInt64}, coef::Vector{Float64})
    id = Ref{Int64}(0)
    check(ccall((:bt_serve_add_plan_client, lib), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ptr{UInt64}, Ptr{UInt64}, Ptr{Float64}, Ref{Int64}),
                s.h, p.h, length(coef), xmask, zmask, coef, id), C_NULL)
    return id[]
end

"""A request: new matrices for the client's parametrised gates (add indices from 0)."""
function submit(s::GPUServer, client::Integer, idx::Vector{Int64}, mats::Vector{<:AbstractMatrix}; seed::Integer=0)
    buf = reduce(vcat, [vec(Matrix{ComplexF64}(m)) for m in mats])
    t = Ref{Int64}(0)
    check(ccall((:bt_serve_submit, lib), Cint,
                (Ptr{Cvoid}, Int64, Cint, Ptr{Int64}, Ptr{ComplexF64}, UInt64, Ref{Int64}),
                s.h, client, length(idx), idx, buf, seed % UInt64, t), C_NULL)
    return t[]
end

"""<H>, latency and service time (seconds) of a request; wait_ms < 0 waits."""
function result(s::GPUServer, ticket::Integer; wait_ms::Integer=-1)
    v, l, t = Ref{Float64}(0.0), Ref{Float64}(0.0), Ref{Float64}(0.0)
    check(ccall((:bt_serve_poll, lib), Cint, (Ptr{Cvoid}, Int64, Int64, Ref{Float64}, Ref{Float64}, Ref{Float64}),
                s.h, ticket, wait_ms, v, l, t), C_NULL)
    return v[], l[], t[]
end

function serve_stats(s::GPUServer)
    done, resident, runs = Ref{Int64}(0), Ref{Int64}(0), Ref{Int64}(0)
    p50, p99, hbm = Ref{Float64}(0.0), Ref{Float64}(0.0), Ref{UInt64}(0)
    check(ccall((:bt_serve_stats, lib), Cint,
                (Ptr{Cvoid}, Ref{Int64}, Ref{Float64}, Ref{Float64}, Ref{Int64}, Ref{UInt64}, Ref{Int64}),
                s.h, done, p50, p99, resident, hbm, runs), C_NULL)
    return (completed=done[], p50_s=p50[], p99_s=p99[], resident=resident[], hbm_used=hbm[], runs=runs[])
end

end # module
