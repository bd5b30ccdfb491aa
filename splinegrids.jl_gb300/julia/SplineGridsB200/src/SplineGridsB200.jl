"""
    SplineGridsB200

`ccall` bindings that make libsplinegrids_b200.so (include/splinegrids_b200.h) the
implementation of SplineGrids.jl's hot path for CUDA-array-backed objects:
`evaluate!(spline_grid)` (src/spline_grid.jl:185-230, spline_eval_kernel),
`evaluate_adjoint!(spline_grid)` (src/adjoint.jl:42-83) and several derivative orders in
one call.  The arrays keep SplineGrids.jl's layout (column-major, Int32 1-based sample
indices, basis tables `eval[ns, d+1, maxd+1]`), so nothing is copied or transposed.

Every primal goes through `evaluate_into!` / `adjoint_into!`, plain functions of device
arrays, so that the differentiation rules (ext/: Enzyme reverse rule, ChainRulesCore
rrule) attach to one place.  Set `ENV["SPLINEGRIDS_B200_LIB"]` to the library's path
before loading (default: `libsplinegrids_b200.so` on the loader path).
"""
module SplineGridsB200

using CUDA
using SplineGrids

const LIB = get(ENV, "SPLINEGRIDS_B200_LIB", "libsplinegrids_b200.so")

const SG_F64, SG_F32, SG_BF16_F32 = Int32(0), Int32(1), Int32(2)
const SG_MAX_NIN = 8

"""Raise the library's message (the reference's wording where it has one) on a status."""
sgcheck(rc) = rc == 0 ? nothing : error(unsafe_string(ccall((:sg_last_error, LIB), Cstring, ())))

dtype_code(::Type{Float64}) = SG_F64
dtype_code(::Type{Float32}) = SG_F32
stream() = CUDA.stream().handle

"""A SplineGrid (or NURBS grid, HasWeights = true) whose eval array lives on the GPU;
Int32 sample indices, as SplineGrids.jl stores them."""
const CuGrid{Nin, Nout, Tv, HW} = SplineGrids.SplineGrid{Nin, Nout, Tv, Int32, <:Any, <:Any, <:Any,
                                                         <:CuArray, HW}

# ------------------------------------------------------------------ grid plans

"""Mirror of `sg_grid_desc`."""
struct GridDesc
    nin::Int32
    nout::Int32
    dtype::Int32
    has_weights::Int32
    n_samples::NTuple{8, Int64}
    n_basis::NTuple{8, Int64}
    degree::NTuple{8, Int32}
    max_derivative_order::NTuple{8, Int32}
    sample_indices::NTuple{8, CuPtr{Int32}}
    basis_eval::NTuple{8, CuPtr{Cvoid}}
end

pad(t, v, T) = ntuple(i -> i <= length(t) ? T(t[i]) : v, SG_MAX_NIN)

function GridDesc(g::SplineGrids.AbstractSplineGrid{Nin, Nout, W, Tv}) where {Nin, Nout, W, Tv}
    ds = g.spline_dimensions
    GridDesc(Nin, Nout, dtype_code(Tv), W ? 1 : 0,
        pad(map(d -> length(d.sample_points), ds), 0, Int64),
        pad(map(SplineGrids.get_n_basis_functions, ds), 0, Int64),
        pad(map(d -> d.degree, ds), 0, Int32),
        pad(map(d -> d.max_derivative_order, ds), 0, Int32),
        pad(map(d -> pointer(d.sample_indices), ds), CU_NULL, CuPtr{Int32}),
        pad(map(d -> reinterpret(CuPtr{Cvoid}, pointer(d.eval)), ds), CU_NULL, CuPtr{Cvoid}))
end

mutable struct Plan
    ptr::Ptr{Cvoid}
end

const PLANS = IdDict{Any, Plan}()

"""The grid's plan (support tables, the separable passes' scratch), created once."""
function plan(g)
    get!(PLANS, g) do
        desc = Ref(GridDesc(g))
        out = Ref{Ptr{Cvoid}}()
        sgcheck(ccall((:sg_grid_plan_create, LIB), Cint,
            (Ref{GridDesc}, CUDA.CUstream, Ref{Ptr{Cvoid}}), desc, stream(), out))
        p = Plan(out[])
        finalizer(q -> ccall((:sg_grid_plan_destroy, LIB), Cvoid, (Ptr{Cvoid},), q.ptr), p)
    end
end

# ------------------------------------------------------------------ primals

"""
    evaluate_into!(eval, grid, control_points, derivative_order)

eval = M(derivative_order) * control_points with the grid's basis tables (and weights,
for a NURBS grid); asynchronous on the task's stream.
"""
function evaluate_into!(eval::CuArray{Tv}, g::SplineGrids.AbstractSplineGrid{Nin, Nout, W, Tv},
        control_points::CuArray{Tv}, derivative_order::NTuple{Nin, Int})::Nothing where {Nin, Nout, W, Tv}
    ord = Int32[derivative_order...]
    w = W ? pointer(g.weights) : CuPtr{Tv}(0)
    sgcheck(ccall((:sg_evaluate, LIB), Cint,
        (Ptr{Cvoid}, Ptr{Int32}, CuPtr{Tv}, CuPtr{Tv}, CuPtr{Tv}, CUDA.CUstream),
        plan(g).ptr, ord, control_points, w, eval, stream()))
    return nothing
end

"""
    adjoint_into!(control_points_bar, grid, eval_bar, derivative_order)

control_points_bar = M(derivative_order)' * eval_bar (overwritten; deterministic gather
form, no atomics).  NURBS grids are refused, as in the reference (src/adjoint.jl:57).
"""
function adjoint_into!(control_points_bar::CuArray{Tv}, g::SplineGrids.AbstractSplineGrid{Nin, Nout, false, Tv},
        eval_bar::CuArray{Tv}, derivative_order::NTuple{Nin, Int})::Nothing where {Nin, Nout, Tv}
    ord = Int32[derivative_order...]
    sgcheck(ccall((:sg_evaluate_adjoint, LIB), Cint,
        (Ptr{Cvoid}, Ptr{Int32}, CuPtr{Tv}, CuPtr{Tv}, CUDA.CUstream),
        plan(g).ptr, ord, eval_bar, control_points_bar, stream()))
    return nothing
end

# ------------------------------------------------------------------ SplineGrids methods

function SplineGrids.evaluate!(g::CuGrid{Nin};
        derivative_order::NTuple{Nin, <:Integer} = ntuple(_ -> 0, Nin),
        control_points = g.control_points, eval::CuArray = g.eval)::Nothing where {Nin}
    SplineGrids.validate_partial_derivatives(g, derivative_order)  # the reference's messages
    evaluate_into!(eval, g, SplineGrids.obtain(control_points), Int.(derivative_order))
    CUDA.synchronize()  # the reference's evaluate! returns after its kernel finished
    return nothing
end

function SplineGrids.evaluate_adjoint!(g::CuGrid{Nin, Nout, Tv, false};
        derivative_order::NTuple{Nin, <:Integer} = ntuple(_ -> 0, Nin),
        control_points = g.control_points, eval::CuArray = g.eval)::Nothing where {Nin, Nout, Tv}
    adjoint_into!(SplineGrids.obtain(control_points), g, eval, Int.(derivative_order))
    CUDA.synchronize()
    return nothing
end

"""
    evaluate_orders!(grid, orders, evals; control_points = grid.control_points)

evaluate! for several derivative orders in one call (sg_evaluate_multi): each shared
prefix of the orders is contracted once; bitwise the results of separate calls.
"""
function evaluate_orders!(g::SplineGrids.AbstractSplineGrid{Nin}, orders::AbstractVector{<:NTuple{Nin, Integer}},
        evals::AbstractVector{<:CuArray}; control_points = g.control_points)::Nothing where {Nin}
    length(orders) == length(evals) || error("one eval array per derivative order is needed")
    ord = Int32[o[k] for o in orders for k in 1:Nin]
    ptrs = [reinterpret(CuPtr{Cvoid}, pointer(e)) for e in evals]
    sgcheck(ccall((:sg_evaluate_multi, LIB), Cint,
        (Ptr{Cvoid}, Int32, Ptr{Int32}, CuPtr{Cvoid}, CuPtr{Cvoid}, Ptr{CuPtr{Cvoid}}, CUDA.CUstream),
        plan(g).ptr, length(orders), ord, SplineGrids.obtain(control_points), CU_NULL, ptrs, stream()))
    CUDA.synchronize()
    return nothing
end

"""
    evaluate_cp(grid, control_points; derivative_order)

Out-of-place evaluation as a function of the control points (a new eval array); the
ChainRulesCore extension gives it an rrule whose pullback is `adjoint_into!`.
"""
function evaluate_cp(g::SplineGrids.AbstractSplineGrid{Nin}, control_points::CuArray;
        derivative_order::NTuple{Nin, Int} = ntuple(_ -> 0, Nin)) where {Nin}
    eval = similar(g.eval)
    evaluate_into!(eval, g, control_points, derivative_order)
    return eval
end

export evaluate_into!, adjoint_into!, evaluate_orders!, evaluate_cp

end # module SplineGridsB200
