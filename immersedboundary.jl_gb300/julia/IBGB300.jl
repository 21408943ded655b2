"""
    IBGB300

Julia binding of libibgb300 (include/ibgb300.h): a `GB300Solver <: AbstractSolver` whose
`advance!` runs the CNAB immersed-boundary step on a GB300 through `ccall`.

    using ImmersedBoundary, IBGB300
    IBGB300.use_gb300!()                 # solve/solve! now build a GB300Solver
    results = solve(prob, (0.0, tf); save=(each_timestep(s -> s.qty.stress[1].CD),))

`use_gb300!()` redefines `ImmersedBoundary.solvertype` for stream-function / CNAB problems,
which is how the reference selects its solver (src/streamfcn/cnab/timestepping.jl:251).
"""
module IBGB300

using ImmersedBoundary
using ImmersedBoundary: AbstractSolver, Problem, fluidof, bodygroup, schemeof, discretize
using ImmersedBoundary.StreamFcn
using ImmersedBoundary.StreamFcn: StreamFcnGrid, BodyStress
using ImmersedBoundary.Fluids: baselevel, nlevels, xycoords, gridstep
using ImmersedBoundary.Bodies: npoints
using ImmersedBoundary.Dynamics: GridFrame, RelativeFrame

const libibgb300 = joinpath(@__DIR__, "..", "libibgb300.so")

const IB_PREC_FP64 = Int32(0)
const IB_PREC_MIXED = Int32(1)
const IB_PREC_MIXED_TC = Int32(2)
const IB_SCHEME_CNAB = Int32(0)
const IB_SCHEME_RKC = Int32(1)
const IB_MOTION_STATIC = Int32(0)
const IB_MOTION_PRESCRIBED = Int32(1)
const IB_PC_SCHUR_REF = Int32(1)
const IB_V2F_AUTO = Int32(0)
const IB_V2F_LEVELS = Int32(1)
const IB_V2F_SEQUENTIAL = Int32(2)

# bodies moving in the grid frame (RigidBody{RelativeFrame}) use ib_advance_kin
moving(bodies) = any(b -> b.frame isa RelativeFrame, bodies)

# mirrors `ib_problem` (natural C alignment; all fields isbits)
struct IbProblem
    nx::Int32
    ny::Int32
    nlevels::Int32
    x0::Float64
    y0::Float64
    h::Float64
    dt::Float64
    beta0::Float64
    beta1::Float64
    re::Float64
    nbodies::Int32
    body_npoints::Ptr{Int32}
    xb::Ptr{Float64}
    ds::Ptr{Float64}
    motion::Int32
    precision::Int32
    device::Int32
    history_capacity::Int32
    refine_sweeps::Int32
    scheme::Int32       # IB_SCHEME_*
    rkc_stages::Int32   # SchemeRKC: 0 picks the fewest stable stages
end

struct IBError <: Exception
    status::Cint
    msg::String
end

function check(status::Cint, handle::Ptr{Cvoid})
    status == 0 && return nothing
    msg = unsafe_string(ccall((:ib_last_error, libibgb300), Cstring, (Ptr{Cvoid},), handle))
    # status 3 is the reference's error("infinite flux") (src/streamfcn/structure-ops.jl:81)
    status == 3 && error("infinite flux")
    throw(IBError(status, msg))
end

mutable struct GB300Solver{P<:Problem} <: AbstractSolver
    prob::P
    handle::Ptr{Cvoid}
    sync::Symbol   # :all (copy state.qty back every step) or :stress (forces only)
    moving::Bool
    kin::Vector{Float64}
end

ImmersedBoundary.problemof(s::GB300Solver) = s.prob

function GB300Solver(prob::Problem, state; precision=IB_PREC_FP64, device=0, sync=:all, precondition=true,
                     vort2flux_order=IB_V2F_AUTO, rkc_stages=0)
    fluid = fluidof(prob)
    grid = discretize(fluid)
    base = baselevel(grid)
    xs, ys = xycoords(base)
    bodies = bodygroup(prob)
    npts = Int32[npoints(b) for b in bodies]
    xb = vcat((b.xb for b in bodies)...)          # nb x 2, column-major
    ds = vcat((b.ds for b in bodies)...)
    scheme = schemeof(prob)
    # SchemeRKC (src/schemes.jl:8-10) carries only dt; the beta fields are CNAB's
    rkc = scheme isa SchemeRKC
    beta = rkc ? (1.5, -0.5) : (scheme.β[1], scheme.β[2])
    mv = moving(bodies)
    handle = Ref{Ptr{Cvoid}}(C_NULL)
    GC.@preserve npts xb ds begin
        p = IbProblem(fluid.domain.nx, fluid.domain.ny, nlevels(grid), first(xs), first(ys),
                      gridstep(base), scheme.dt, beta[1], beta[2], fluid.Re,
                      length(npts), pointer(npts), pointer(xb), pointer(ds),
                      mv ? IB_MOTION_PRESCRIBED : IB_MOTION_STATIC, precision, device, 4096, 0,
                      rkc ? IB_SCHEME_RKC : IB_SCHEME_CNAB, rkc_stages)
        st = ccall((:ib_create, libibgb300), Cint, (Ref{IbProblem}, Ref{Ptr{Cvoid}}), p, handle)
        check(st, C_NULL)
    end
    s = GB300Solver(prob, handle[], sync, mv, zeros(6 * length(npts)))
    finalizer(x -> ccall((:ib_destroy, libibgb300), Cint, (Ptr{Cvoid},), x.handle), s)
    if mv && precondition
        check(ccall((:ib_set_cg_preconditioner, libibgb300), Cint, (Ptr{Cvoid}, Int32, Int32),
                    s.handle, IB_PC_SCHUR_REF, 0), s.handle)
    end
    # mixed precision: all levels of Vort2Flux in one batch, or the reference's level order
    check(ccall((:ib_set_vort2flux_order, libibgb300), Cint, (Ptr{Cvoid}, Int32), s.handle, vort2flux_order),
          s.handle)
    push_state!(s, state)
    return s
end

"Upload `state` (Γ, q, ψ, nonlin, Fb, t) to the device."
function push_state!(s::GB300Solver, state)
    qty = state.qty
    st = ccall((:ib_set_state, libibgb300), Cint,
               (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
                Ptr{Float64}, Cdouble),
               s.handle, qty.Γ, qty.q, qty.ψ, state.nonlin[1], state.nonlin[2], qty.Fb, state.t)
    check(st, s.handle)
end

"Copy the device state back into `state` (what `advance!` leaves in state.qty)."
function pull_state!(s::GB300Solver, state)
    qty = state.qty
    tref = Ref{Cdouble}(0.0)
    st = ccall((:ib_get_state, libibgb300), Cint,
               (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
                Ptr{Float64}, Ref{Cdouble}),
               s.handle, qty.Γ, qty.q, qty.ψ, state.nonlin[1], state.nonlin[2], qty.Fb, tref)
    check(st, s.handle)
end

function pull_stress!(s::GB300Solver, state)
    bodies = bodygroup(s.prob)
    nbod = length(bodies)
    cd = zeros(nbod)
    cl = zeros(nbod)
    fb = zeros(2 * npoints(bodies))
    st = ccall((:ib_get_stress, libibgb300), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
               s.handle, cd, cl, fb)
    check(st, s.handle)
    i = 0
    for (k, b) in enumerate(bodies)
        n = npoints(b)
        blk = reshape(fb[(2i+1):(2i+2n)], n, 2)
        state.qty.stress[k] = BodyStress(blk, cd[k], cl[k])
        i += n
    end
end

"`advance!(state, solver, t)`: src/streamfcn/cnab/timestepping.jl:253-290 on the GPU."
function ImmersedBoundary.advance!(state, solver::GB300Solver, t::Float64)
    u, v = fluidof(solver.prob).freestream(t)
    # a grid translating with a RelativeFrame of the lab frame sees the freestream minus its
    # velocity (base_flux! for a moving grid, the reference's TODO at fluid-ops.jl:419)
    gframe = fluidof(solver.prob).domain.frame
    if gframe isa RelativeFrame
        # a rotating grid would add fictitious terms the stream-function step does not model
        (gframe.θ(t) == 0 && gframe.Ω(t) == 0) || error("a rotating grid frame is not supported")
        gv = gframe.v(t)
        u, v = u - gv[1], v - gv[2]
    end
    st = if solver.moving
        # update_bodies! (src/bodies/body-points.jl:52-68): the frame closures at t, per body
        for (k, b) in enumerate(bodygroup(solver.prob))
            f = b.frame
            r, vel, θ, Ω = f isa RelativeFrame ? (f.r(t), f.v(t), f.θ(t), f.Ω(t)) : ((0.0, 0.0), (0.0, 0.0), 0.0, 0.0)
            solver.kin[6k-5:6k] .= (r[1], r[2], vel[1], vel[2], θ, Ω)
        end
        ccall((:ib_advance_kin, libibgb300), Cint, (Ptr{Cvoid}, Cdouble, Cdouble, Cdouble, Ptr{Float64}),
              solver.handle, t, u, v, solver.kin)
    else
        ccall((:ib_advance, libibgb300), Cint, (Ptr{Cvoid}, Cdouble, Cdouble, Cdouble),
              solver.handle, t, u, v)
    end
    check(st, solver.handle)
    solver.sync === :all && pull_state!(solver, state)
    pull_stress!(solver, state)
    state.t = t
    return nothing
end

"""
Make `solve` / `solve!` use the GB300 solver for stream-function problems: CNAB, and
SchemeRKC, which the reference declares without a state or solver type (its state here is
CNAB's: `qty`, `nonlin` (unused by RKC) and `t`).
"""
function use_gb300!(; precision=IB_PREC_FP64, device=0, sync=:all)
    @eval function ImmersedBoundary.solvertype(
        ::Problem{<:StreamFcnFluid{<:StreamFcnGrid},<:Any,<:Union{SchemeCNAB,SchemeRKC}}
    )
        return (prob, state) -> GB300Solver(prob, state; precision=$precision, device=$device, sync=$(QuoteNode(sync)))
    end
    @eval ImmersedBoundary.statetype(::Problem{<:StreamFcnFluid{<:StreamFcnGrid},<:Any,<:SchemeRKC}) =
        ImmersedBoundary.StreamFcn.CNAB.State
    return nothing
end

"Write the solver's state to a checkpoint file (`ib_checkpoint_save`)."
function save_checkpoint(s::GB300Solver, path::AbstractString)
    check(ccall((:ib_checkpoint_save, libibgb300), Cint, (Ptr{Cvoid}, Cstring), s.handle, path), s.handle)
end

"Restore the solver from a checkpoint file of the same problem and refresh `state` from it."
function load_checkpoint!(s::GB300Solver, state, path::AbstractString)
    check(ccall((:ib_checkpoint_load, libibgb300), Cint, (Ptr{Cvoid}, Cstring), s.handle, path), s.handle)
    pull_state!(s, state)
    pull_stress!(s, state)
    tref = Ref{Cdouble}(0.0)
    check(ccall((:ib_get_state, libibgb300), Cint,
                (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
                 Ptr{Float64}, Ref{Cdouble}),
                s.handle, C_NULL, C_NULL, C_NULL, C_NULL, C_NULL, C_NULL, tref), s.handle)
    state.t = tref[]
    return state
end

end # module
