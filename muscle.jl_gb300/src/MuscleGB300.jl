"""
    MuscleGB300

A Muscle.jl backend for device-resident tensors on NVIDIA GB300 (sm_103a).
Loading it routes `binary_einsum`, `binary_einsum!`, `unary_einsum`,
`unary_einsum!`, `hadamard` and `hadamard!` on CuArray-backed tensors to
`BackendGB300` by adding methods beside the rule tables of
src/Operations/binary_einsum.jl:20-31, src/Operations/unary_einsum.jl:20-24
and src/Operations/hadamard.jl:4-5 (none is replaced); the methods `ccall`
into `libmuscle_gb300.so` (C ABI in include/muscle_gb300.h).
`with_backend(f, BackendGB300(...))` selects a form explicitly. `Group` runs
many independent contractions (a PEPS sweep's site pairs) as a few batched
launches on one stream; `block_einsum` splits one contraction into blocks
and runs them as such a group. `Server` is the serving loop: contractions submitted
as they arrive, admitted against a device-memory budget and batched onto
several streams.
"""
module MuscleGB300

using CUDA
using Muscle
using Muscle: Backend, DomainCUDA, Index, Tensor, inds

export BackendGB300, Server, submit!, Group, execute!, block_einsum

const libmgb = get(ENV, "MUSCLE_GB300_LIB", joinpath(@__DIR__, "..", "lib", "libmuscle_gb300.so"))

const FORMS = Dict(:auto => Cint(0), :plain => Cint(1), :ozaki => Cint(2), :bf16x3 => Cint(3))

"""
    BackendGB300(; form=:auto, slices=0)

`form`: `:auto` (Ozaki emulation for Float64/ComplexF64 results, BF16x3 for
Float32/ComplexF32), `:plain` (native FP64 DMMA / FP32 FFMA), `:ozaki`,
`:bf16x3`. `slices`: Ozaki slice count (3..8; 0: chosen on the device per
call, the fewest slices whose error estimate meets a 1e-13 relative target).
"""
struct BackendGB300 <: Backend
    form::Cint
    slices::Cint
end
BackendGB300(; form::Symbol=:auto, slices::Integer=0) = BackendGB300(FORMS[form], Cint(slices))

# mirrors `mgb_tensor_desc`
struct TensorDesc
    dtype::Cint
    rank::Cint
    modes::Ptr{Cint}
    extents::Ptr{Int64}
    strides::Ptr{Int64}
end

dtype_code(::Type{Float32}) = Cint(0)
dtype_code(::Type{Float64}) = Cint(1)
dtype_code(::Type{ComplexF32}) = Cint(2)
dtype_code(::Type{ComplexF64}) = Cint(3)
dtype_code(::Type{T}) where {T} = throw(ArgumentError("eltype $T is not supported by BackendGB300"))

function check(status::Cint)
    status == 0 && return nothing
    msg = unsafe_string(ccall((:mgb_last_error, libmgb), Cstring, ()))
    status == 1 && throw(ArgumentError(msg))
    status == 2 && throw(DimensionMismatch(msg))
    status == 3 && throw(ArgumentError(msg))
    status == 7 && throw(CUDA.OutOfGPUMemoryError(0))
    error("libmuscle_gb300 status $status: $msg")
end

# labels -> integer modes by first appearance (ext/MuscleCUDAExt.jl:24-27)
function modemap(tensors...)
    m = Dict{Index,Cint}()
    for t in tensors, i in inds(t)
        haskey(m, i) || (m[i] = Cint(length(m)))
    end
    m
end

# arrays kept alive by the caller with GC.@preserve
descarrays(t::Tensor, m) = (Cint[m[i] for i in inds(t)], Int64[size(t)...], Int64[strides(parent(t))...])
function desc(t::Tensor, arrs)
    modes, ext, str = arrs
    TensorDesc(dtype_code(eltype(t)), Cint(ndims(t)), pointer(modes), pointer(ext), pointer(str))
end

function with_plan(f, create)
    plan = Ref{Ptr{Cvoid}}(C_NULL)
    check(create(plan))
    try
        f(plan[])
    finally
        ccall((:mgb_plan_destroy, libmgb), Cint, (Ptr{Cvoid},), plan[])
    end
end

function workspace(plan)
    bytes = Ref{UInt64}(0)
    check(ccall((:mgb_plan_workspace_size, libmgb), Cint, (Ptr{Cvoid}, Ref{UInt64}), plan, bytes))
    bytes[] == 0 ? (CU_NULL, UInt64(0)) : (CuArray{UInt8}(undef, bytes[]), bytes[])
end

# binary_einsum(::Backend, inds_c, a, b)  (src/Operations/binary_einsum.jl:50)
function Muscle.binary_einsum(be::BackendGB300, inds_c, a::Tensor, b::Tensor)
    sizes = Dict{Index,Int}()
    for t in (a, b), (i, s) in zip(inds(t), size(t))
        sizes[i] = s
    end
    T = Base.promote_eltype(a, b)
    c = Tensor(similar(parent(a), T, Tuple(sizes[i] for i in inds_c)), collect(inds_c))
    return Muscle.binary_einsum!(be, c, a, b)
end

# binary_einsum!(::Backend, c, a, b)  (src/Operations/binary_einsum.jl:68)
function Muscle.binary_einsum!(be::BackendGB300, c::Tensor, a::Tensor, b::Tensor)
    m = modemap(a, b, c)
    aa, ab, ac = descarrays(a, m), descarrays(b, m), descarrays(c, m)
    GC.@preserve aa ab ac begin
        da, db, dc = Ref(desc(a, aa)), Ref(desc(b, ab)), Ref(desc(c, ac))
        with_plan(p -> ccall((:mgb_contraction_plan, libmgb), Cint,
                             (Ptr{Ptr{Cvoid}}, Ref{TensorDesc}, Ref{TensorDesc}, Ref{TensorDesc}, Cint, Cint),
                             p, da, db, dc, be.form, be.slices)) do plan
            ws, nbytes = workspace(plan)
            check(ccall((:mgb_contract, libmgb), Cint,
                        (Ptr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, UInt64, CUDA.CUstream),
                        plan, parent(a), parent(b), parent(c), ws, nbytes, CUDA.stream()))
        end
    end
    return c
end

# unary_einsum(::Backend, inds_y, x)  (src/Operations/unary_einsum.jl:35)
function Muscle.unary_einsum(be::BackendGB300, inds_y, x::Tensor)
    y = Tensor(similar(parent(x), Tuple(size(x, i) for i in inds_y)), collect(inds_y))
    return Muscle.unary_einsum!(be, y, x)
end

# unary_einsum!(::Backend, y, x)  (src/Operations/unary_einsum.jl:44)
function Muscle.unary_einsum!(::BackendGB300, y::Tensor, x::Tensor)
    m = modemap(x, y)
    ax, ay = descarrays(x, m), descarrays(y, m)
    GC.@preserve ax ay begin
        dx, dy = Ref(desc(x, ax)), Ref(desc(y, ay))
        with_plan(p -> ccall((:mgb_unary_plan, libmgb), Cint,
                             (Ptr{Ptr{Cvoid}}, Ref{TensorDesc}, Ref{TensorDesc}), p, dx, dy)) do plan
            check(ccall((:mgb_unary, libmgb), Cint,
                        (Ptr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, UInt64, CUDA.CUstream),
                        plan, parent(x), parent(y), CU_NULL, UInt64(0), CUDA.stream()))
        end
    end
    return y
end

# hadamard(::Backend, a, b)  (src/Operations/hadamard.jl:34-40): c has a's
# labels and a's element type
function Muscle.hadamard(be::BackendGB300, a::Tensor, b::Tensor)
    ndims(a) >= ndims(b) || return Muscle.hadamard(be, b, a)
    c = Tensor(similar(parent(a)), collect(inds(a)))
    return Muscle.hadamard!(be, c, a, b)
end

# hadamard!(::Backend, c, a, b)  (src/Operations/hadamard.jl:42-77)
function Muscle.hadamard!(be::BackendGB300, c::Tensor, a::Tensor, b::Tensor)
    ndims(a) >= ndims(b) || return Muscle.hadamard!(be, c, b, a)
    m = modemap(a, b, c)
    aa, ab, ac = descarrays(a, m), descarrays(b, m), descarrays(c, m)
    GC.@preserve aa ab ac begin
        da, db, dc = Ref(desc(a, aa)), Ref(desc(b, ab)), Ref(desc(c, ac))
        check(ccall((:mgb_hadamard, libmgb), Cint,
                    (Ref{TensorDesc}, Ref{TensorDesc}, Ref{TensorDesc}, CuPtr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid},
                     CUDA.CUstream),
                    da, db, dc, parent(a), parent(b), parent(c), CUDA.stream()))
    end
    return c
end

# ---------------------------------------------------------------------------
# Serving loop (mgb_server_*): contractions submitted as they arrive, admitted
# against a device-memory byte budget and batched onto several streams by the
# library's scheduler thread.

"""
    Server(budget_bytes; streams=4, max_batch=256)

A request loop on the current device. `submit!` hands it a contraction
`c = a * b` (labels as in `binary_einsum!`); `wait` blocks for its result.
The tensors must stay alive until `wait` returns for their ticket.
"""
mutable struct Server
    handle::Ptr{Cvoid}
    plans::Dict{Int64,Ptr{Cvoid}}  # ticket -> plan, destroyed once waited for
end

function Server(budget_bytes::Integer; streams::Integer=4, max_batch::Integer=256)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:mgb_server_create, libmgb), Cint, (Ptr{Ptr{Cvoid}}, UInt64, Cint, Cint),
                h, UInt64(budget_bytes), Cint(streams), Cint(max_batch)))
    srv = Server(h[], Dict{Int64,Ptr{Cvoid}}())
    finalizer(close, srv)
    return srv
end

function submit!(srv::Server, c::Tensor, a::Tensor, b::Tensor; backend::BackendGB300=BackendGB300())
    m = modemap(a, b, c)
    aa, ab, ac = descarrays(a, m), descarrays(b, m), descarrays(c, m)
    plan = Ref{Ptr{Cvoid}}(C_NULL)
    GC.@preserve aa ab ac begin
        da, db, dc = Ref(desc(a, aa)), Ref(desc(b, ab)), Ref(desc(c, ac))
        check(ccall((:mgb_contraction_plan, libmgb), Cint,
                    (Ptr{Ptr{Cvoid}}, Ref{TensorDesc}, Ref{TensorDesc}, Ref{TensorDesc}, Cint, Cint),
                    plan, da, db, dc, backend.form, backend.slices))
    end
    resident = UInt64(sizeof(parent(a)) + sizeof(parent(b)) + sizeof(parent(c)))
    ticket = Ref{Int64}(0)
    check(ccall((:mgb_server_submit, libmgb), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, UInt64, CUDA.CUstream, Ref{Int64}),
                srv.handle, plan[], parent(a), parent(b), parent(c), resident, CUDA.stream(), ticket))
    srv.plans[ticket[]] = plan[]
    return ticket[]
end

function Base.wait(srv::Server, ticket::Integer; timeout::Real=-1)
    status = Ref{Cint}(0)
    check(ccall((:mgb_server_wait, libmgb), Cint, (Ptr{Cvoid}, Int64, Cdouble, Ref{Cint}),
                srv.handle, Int64(ticket), Cdouble(timeout), status))
    plan = pop!(srv.plans, Int64(ticket), C_NULL)
    plan == C_NULL || ccall((:mgb_plan_destroy, libmgb), Cint, (Ptr{Cvoid},), plan)
    check(status[])
    return nothing
end

function Base.close(srv::Server)
    srv.handle == C_NULL && return nothing
    ccall((:mgb_server_destroy, libmgb), Cint, (Ptr{Cvoid},), srv.handle)
    for plan in values(srv.plans)
        ccall((:mgb_plan_destroy, libmgb), Cint, (Ptr{Cvoid},), plan)
    end
    empty!(srv.plans)
    srv.handle = C_NULL
    return nothing
end

# ---------------------------------------------------------------------------
# Grouped contractions (mgb_group_*): independent c = a * b on one stream.
# Members with equal plans (same shapes, strides, element types and form)
# share one plan handle and run as one batched launch per kernel; the
# emulated buckets' tensor-core work runs as one persistent launch per kernel
# variant. ext/MuscleDaggerExt/binary_einsum.jl:64-119 runs such pairs as
# separate tasks.

devptr(t::Tensor) = Ptr{Cvoid}(reinterpret(UInt64, pointer(parent(t))))

"""
    Group(items; backend=BackendGB300())

`items`: `(c, a, b)` tensor triples, labels as in `binary_einsum!`.
`execute!(g)` computes every `c` on the current stream. After one
`execute!`, the call can be captured into a CUDA graph and replayed; the
device state it launches with stays valid until `close(g)`. The tensors must
stay alive, at the same addresses, as long as the group.
"""
mutable struct Group
    handle::Ptr{Cvoid}
    plans::Vector{Ptr{Cvoid}}  # distinct plans, destroyed with the group
    items::Vector{Any}
    workspace::Union{CuArray{UInt8,1},Nothing}
    nbytes::UInt64
end

function Group(items; backend::BackendGB300=BackendGB300())
    cache = Dict{Any,Ptr{Cvoid}}()
    members = Ptr{Cvoid}[]
    g = Group(C_NULL, Ptr{Cvoid}[], collect(Any, items), nothing, UInt64(0))
    finalizer(close, g)
    for (c, a, b) in g.items
        m = modemap(a, b, c)
        aa, ab, ac = descarrays(a, m), descarrays(b, m), descarrays(c, m)
        key = (eltype(a), eltype(b), eltype(c), aa, ab, ac)
        plan = get(cache, key, C_NULL)
        if plan == C_NULL
            ref = Ref{Ptr{Cvoid}}(C_NULL)
            GC.@preserve aa ab ac begin
                da, db, dc = Ref(desc(a, aa)), Ref(desc(b, ab)), Ref(desc(c, ac))
                check(ccall((:mgb_contraction_plan, libmgb), Cint,
                            (Ptr{Ptr{Cvoid}}, Ref{TensorDesc}, Ref{TensorDesc}, Ref{TensorDesc}, Cint, Cint),
                            ref, da, db, dc, backend.form, backend.slices))
            end
            plan = cache[key] = ref[]
            push!(g.plans, plan)
        end
        push!(members, plan)
    end
    A = Ptr{Cvoid}[devptr(a) for (c, a, b) in g.items]
    B = Ptr{Cvoid}[devptr(b) for (c, a, b) in g.items]
    C = Ptr{Cvoid}[devptr(c) for (c, a, b) in g.items]
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:mgb_group_create, libmgb), Cint,
                (Ptr{Ptr{Cvoid}}, Ptr{Ptr{Cvoid}}, Cint, Ptr{Ptr{Cvoid}}, Ptr{Ptr{Cvoid}}, Ptr{Ptr{Cvoid}}),
                h, members, Cint(length(members)), A, B, C))
    g.handle = h[]
    bytes = Ref{UInt64}(0)
    check(ccall((:mgb_group_workspace_size, libmgb), Cint, (Ptr{Cvoid}, Ref{UInt64}), g.handle, bytes))
    g.nbytes = bytes[]
    g.workspace = bytes[] == 0 ? nothing : CuArray{UInt8}(undef, bytes[])
    return g
end

function execute!(g::Group)
    ws = g.workspace === nothing ? CU_NULL : pointer(g.workspace)
    check(ccall((:mgb_group_execute, libmgb), Cint, (Ptr{Cvoid}, CuPtr{Cvoid}, UInt64, CUDA.CUstream),
                g.handle, ws, g.nbytes, CUDA.stream()))
    return g
end

"""
    set_bands!(g, bands)

Rasterisation band per member: an index 0..5 into {1, 2, 3, 4, 8, 16} row
tiles (any other value: the library's default). A schedule choice only.
"""
function set_bands!(g::Group, bands::AbstractVector{<:Integer})
    length(bands) == length(g.items) || throw(ArgumentError("one band per member"))
    check(ccall((:mgb_group_set_tiles, libmgb), Cint, (Ptr{Cvoid}, Ptr{Cint}), g.handle, Cint.(bands)))
    return g
end

"""
    block_einsum(a, b, blocksize; out=nothing, rank=0, world=1, backend=BackendGB300())

Block-partitioned contraction, the decomposition of
ext/MuscleDaggerExt/binary_einsum.jl:64-119 on device tensors: `blocksize`
maps labels to block sizes (each must divide its extent; other labels are one
block). Every block pair runs as a member of one `Group` (views, no copies);
the partial products of an output block, one per block of the contracted
labels, are stacked along one extra label and summed by `unary_einsum!` (the
reference's `treereduce(AddComputeOp, ...)`). With `world > 1` only the output
blocks of replica `rank` are written, into a zero output, dealt largest work
first to the least loaded replica.
"""
function block_einsum(a::Tensor, b::Tensor, blocksize::AbstractDict; out=nothing, rank::Integer=0,
                      world::Integer=1, backend::BackendGB300=BackendGB300())
    ia, ib = collect(inds(a)), collect(inds(b))
    ic = out === nothing ? setdiff(union(ia, ib), intersect(ia, ib)) : collect(out)
    ext = Dict{Index,Int}()
    for (labs, t) in ((ia, a), (ib, b)), (k, i) in enumerate(labs)
        haskey(ext, i) && ext[i] != size(t, k) && throw(DimensionMismatch("label $i has different extents"))
        ext[i] = size(t, k)
    end
    all(i -> haskey(ext, i), ic) || throw(ArgumentError("ic must be a subset of ia ∪ ib"))
    all(i -> haskey(ext, i), keys(blocksize)) || throw(ArgumentError("block size of a label of neither operand"))
    bs = Dict(i => get(blocksize, i, ext[i]) for i in keys(ext))
    for (i, s) in bs
        (s > 0 && ext[i] % s == 0) || throw(ArgumentError("block size $s of label $i must divide $(ext[i])"))
    end
    0 <= rank < world || throw(ArgumentError("rank out of range"))
    nb(i) = ext[i] ÷ bs[i]
    rng(labels, co) = Tuple(haskey(co, i) ? ((co[i] * bs[i] + 1):((co[i] + 1) * bs[i])) : Colon() for i in labels)
    sums = setdiff(union(ia, ib), ic)
    T = promote_type(eltype(a), eltype(b))
    C = Tensor(world > 1 ? CUDA.zeros(T, (ext[i] for i in ic)...) : CuArray{T}(undef, (ext[i] for i in ic)...), ic)
    # output blocks, equal work each: dealt round robin over the replicas
    outs = vec(collect(Iterators.product((0:(nb(i) - 1) for i in ic)...)))
    mine = [o for (k, o) in enumerate(outs) if (k - 1) % world == rank]
    ksets = vec(collect(Iterators.product((0:(nb(i) - 1) for i in sums)...)))
    items, reductions, part = Any[], Any[], Index(gensym(:block_part))
    for o in mine
        co = Dict(zip(ic, o))
        cview = Tensor(view(parent(C), rng(ic, co)...), ic)
        pairs = map(ksets) do kc
            c2 = merge(co, Dict(zip(sums, kc)))
            (Tensor(view(parent(a), rng(ia, c2)...), ia), Tensor(view(parent(b), rng(ib, c2)...), ib))
        end
        if length(pairs) == 1
            push!(items, (cview, pairs[1]...))
        else
            P = CuArray{T}(undef, (bs[i] for i in ic)..., length(pairs))
            for (k, (va, vb)) in enumerate(pairs)
                push!(items, (Tensor(view(P, ntuple(_ -> Colon(), length(ic))..., k), ic), va, vb))
            end
            push!(reductions, (cview, Tensor(P, [ic; part])))
        end
    end
    if !isempty(items)
        g = Group(items; backend)
        execute!(g)
        for (y, x) in reductions
            Muscle.unary_einsum!(backend, y, x)
        end
        CUDA.synchronize()
        close(g)
    end
    return C
end

function Base.close(g::Group)
    if g.handle != C_NULL
        ccall((:mgb_group_destroy, libmgb), Cint, (Ptr{Cvoid},), g.handle)
        g.handle = C_NULL
    end
    for plan in g.plans
        ccall((:mgb_plan_destroy, libmgb), Cint, (Ptr{Cvoid},), plan)
    end
    empty!(g.plans)
    return nothing
end

# ---------------------------------------------------------------------------
# tensor_svd_thin (src/Operations/tensor_svd.jl:98-125) and simple_update
# (src/Operations/simple_update.jl:35-82) on the device: contractions and
# absorbs through the library, the thin SVD through mgb_svd (one-sided Jacobi)

# permutedims by labels (src/Tensor.jl:316-319) through mgb_permute: a dense
# column-major copy with labels `to`
function permute_device(t::Tensor, to)
    y = Tensor(similar(parent(t), Tuple(size(t, i) for i in to)), collect(to))
    m = modemap(t)
    at, ay = descarrays(t, m), descarrays(y, m)
    GC.@preserve at ay begin
        check(ccall((:mgb_permute, libmgb), Cint,
                    (Ref{TensorDesc}, Ref{TensorDesc}, CuPtr{Cvoid}, CuPtr{Cvoid}, CUDA.CUstream),
                    Ref(desc(t, at)), Ref(desc(y, ay)), parent(t), parent(y), CUDA.stream()))
    end
    return y
end

const SVD_NORMALIZE, SVD_CONJ_V, SVD_SQRT_S = Cint(1), Cint(2), Cint(4)

function svd_device(::BackendGB300, x::Tensor, inds_u, inds_v, ind_s; keep::Integer=0, flags::Cint=SVD_CONJ_V)
    T = eltype(x)
    T in (Float64, ComplexF64) || throw(ArgumentError("tensor_svd_thin on the device: Float64 or ComplexF64"))
    xm = permute_device(x, [inds_u; inds_v])
    su, sv = [size(x, i) for i in inds_u], [size(x, i) for i in inds_v]
    m, n = prod(su), prod(sv)
    k = min(m, n)
    keep = keep <= 0 ? k : min(keep, k)
    bytes = Ref{UInt64}(0)
    check(ccall((:mgb_svd_workspace_size, libmgb), Cint, (Cint, Int64, Int64, Ref{UInt64}), dtype_code(T), m, n, bytes))
    ws = CuArray{UInt8}(undef, max(bytes[], 1))
    U = similar(parent(x), T, su..., keep)
    s = similar(parent(x), Float64, keep)
    V = similar(parent(x), T, sv..., keep)
    check(ccall((:mgb_svd, libmgb), Cint,
                (Cint, Int64, Int64, CuPtr{Cvoid}, Int64, CuPtr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, Cint, Cint,
                 CuPtr{Cvoid}, UInt64, CUDA.CUstream),
                dtype_code(T), m, n, parent(xm), max(m, 1), U, s, V, Cint(keep), flags, ws, bytes[], CUDA.stream()))
    return Tensor(U, [inds_u; ind_s]), Tensor(s, [ind_s]), Tensor(V, [inds_v; ind_s])
end

function Muscle.tensor_svd_thin(be::BackendGB300, A::Tensor; inds_u=(), inds_v=(), ind_s=Index(gensym(:vind)),
                                inplace=false, kwargs...)
    inds_u, inds_v = Muscle.factorinds(inds(A), inds_u, inds_v)
    return svd_device(be, A, collect(inds_u), collect(inds_v), ind_s)
end

function Muscle.simple_update(be::BackendGB300, A::Tensor, ind_physical_a::Index, B::Tensor, ind_physical_b::Index,
                              ind_bond_ab::Index, G::Tensor, ind_physical_g_a::Index, ind_physical_g_b::Index;
                              normalize::Bool=false, absorb::Muscle.AbsorbBehavior=Muscle.DontAbsorb(),
                              atol::Float64=0.0, rtol::Float64=0.0, maxdim=nothing)
    Θ = Muscle.with_backend(be) do
        Muscle.binary_einsum(Muscle.binary_einsum(A, B; dims=[ind_bond_ab]), G; dims=[ind_physical_a, ind_physical_b])
    end
    Θ = replace(Θ, ind_physical_g_a => ind_physical_a, ind_physical_g_b => ind_physical_b)
    inds_u = setdiff(inds(A), [ind_bond_ab])
    inds_v = setdiff(inds(B), [ind_bond_ab])
    flags = SVD_CONJ_V | (normalize ? SVD_NORMALIZE : Cint(0)) | (absorb isa Muscle.AbsorbEqually ? SVD_SQRT_S : Cint(0))
    U, s, V = svd_device(be, Θ, inds_u, inds_v, ind_bond_ab; keep=something(maxdim, 0), flags)
    absorb isa Muscle.DontAbsorb && return U, s, V
    absorb isa Muscle.AbsorbV || Muscle.hadamard!(be, U, U, s)
    absorb isa Muscle.AbsorbU || Muscle.hadamard!(be, V, V, s)
    return U, V
end

# ---------------------------------------------------------------------------
# Routing device-resident operands here without replacing any Muscle method.
#  * binary_einsum / binary_einsum!: the rules of src/Operations/binary_einsum.jl:21,30
#    select BackendCuTENSOR, whose CUDA extension defines only 6-argument
#    methods (ext/MuscleCUDAExt.jl:10,22) while the front-ends call the
#    4-argument ones (src/Operations/binary_einsum.jl:50,68). These are those
#    missing 4-argument methods, for tensors whose parent is a CuArray.
#  * unary_einsum / unary_einsum!: the rules select BackendOMEinsum
#    (src/Operations/unary_einsum.jl:21,24); methods for CuArray-backed tensors
#    are more specific than the extension's generic ones
#    (ext/MuscleOMEinsumExt.jl:25,31).
#  * hadamard / hadamard!: rules for (DomainCUDA, ...) operands are more
#    specific than the generic (Domain, ...) rules of src/Operations/hadamard.jl:4-5.
#  * simple_update: the rule selects BackendCuTensorNet
#    (src/Operations/simple_update.jl:5); a method for CuArray-backed tensors is
#    more specific than the extension's (ext/MusclecuTensorNetExt.jl:13).
# Every definition below adds a method; none overwrites one, so loading the
# package is enough and precompilation stays clean.
const CuTensor = Tensor{<:Any,<:Any,<:CuArray}

Muscle.binary_einsum(::Muscle.BackendCuTENSOR, inds_c, a::CuTensor, b::CuTensor) =
    Muscle.binary_einsum(BackendGB300(), inds_c, a, b)
Muscle.binary_einsum!(::Muscle.BackendCuTENSOR, c::CuTensor, a::CuTensor, b::CuTensor) =
    Muscle.binary_einsum!(BackendGB300(), c, a, b)
Muscle.unary_einsum(::Muscle.BackendOMEinsum, inds_y, x::CuTensor) = Muscle.unary_einsum(BackendGB300(), inds_y, x)
Muscle.unary_einsum!(::Muscle.BackendOMEinsum, y::CuTensor, x::CuTensor) = Muscle.unary_einsum!(BackendGB300(), y, x)
Muscle.simple_update(::Muscle.BackendCuTensorNet, A::CuTensor, pa::Index, B::CuTensor, pb::Index, bond::Index,
                     G::CuTensor, ga::Index, gb::Index; kwargs...) =
    Muscle.simple_update(BackendGB300(), A, pa, B, pb, bond, G, ga, gb; kwargs...)
Muscle.choose_backend_rule(::typeof(Muscle.hadamard), ::Muscle.DomainCUDA, ::Muscle.DomainCUDA) = BackendGB300()
Muscle.choose_backend_rule(::typeof(Muscle.hadamard!), ::Muscle.DomainCUDA, ::Muscle.DomainCUDA, ::Muscle.DomainCUDA) =
    BackendGB300()

"""
    MuscleGB300.enable!()

Checks that `libmuscle_gb300.so` loads and returns its version string. The
routing of device-resident operands to `BackendGB300` is active as soon as
the package is loaded (methods added next to Muscle's rules, none replaced);
`with_backend(f, BackendGB300(form, slices))` selects a form explicitly.
"""
function enable!()
    return unsafe_string(ccall((:mgb_version, libmgb), Cstring, ()))
end

end # module
