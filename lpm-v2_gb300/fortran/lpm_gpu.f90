module LpmGpuModule
!> @file lpm_gpu.f90
!> iso_c_binding interface to liblpm_gpu.so, the GB300 direct-sum library.
!>
!> Each routine here is a drop-in body for one lpm-v2 direct sum.  The arrays are passed by
!> base address (Fortran arrays are contiguous), the target block of this MPI rank is passed
!> as the 1-based indexStart/indexEnd of MPISetup, and a non-zero status is reported through
!> the module's Logger at ERROR level (which also clears testPass, as the reference's own
!> error reporting does).  The MPI_BCAST re-replication after each sum is unchanged.
!>
!> Build: gfortran -c lpm_gpu.f90 (after the lpm-v2 modules), link with -llpm_gpu.
use iso_c_binding
use NumberKindsModule
use LoggerModule

implicit none
private

public :: LPM_MODE_FP64, LPM_MODE_FP32C, LPM_PSE_K8_GEODESIC, LPM_PSE_GAUSS_CHORD, LPM_PSE_K8_CHORD
public :: GpuMask, GpuBVESphereVelocity, GpuPlanarVelocity, GpuPSESphereLaplacian, GpuStatusCheck
public :: lpm_bve_velocity, lpm_bve_set_velocity_from_vorticity, lpm_plane_velocity
public :: lpm_pse_sphere_laplacian, lpm_pse_plane_laplacian, lpm_bve_stream_functions
public :: lpm_plane_stream_function, lpm_last_error_string
public :: lpm_pse_sphere_gradient, lpm_pse_sphere_divergence
public :: lpm_pse_plane_gradient, lpm_pse_plane_second_partials, lpm_pse_plane_double_dot
public :: lpm_pse_sphere_double_dot, lpm_pse_interpolate_scalar
public :: lpm_swe_plane_rhs_integrals, lpm_swe_sphere_rhs_integrals
public :: lpm_beta_plane_velocity, lpm_beta_plane_stream_functions, lpm_bve_solver_remesh
public :: lpm_plane_solver_remesh
public :: lpm_bve_solver_create, lpm_bve_timestep, lpm_bve_get_state, lpm_bve_set_state
public :: lpm_bve_diagnostics, lpm_bve_solver_stream_functions, lpm_bve_solver_destroy
public :: lpm_plane_solver_create, lpm_plane_timestep, lpm_plane_get_state, lpm_plane_diagnostics
public :: lpm_plane_solver_destroy
public :: lpm_ensemble_create, lpm_ensemble_timestep, lpm_ensemble_velocity, lpm_ensemble_get_state
public :: lpm_ensemble_destroy, lpm_bve_kernel_timing, lpm_bve_solver_set_timing, lpm_version
public :: lpm_ensemble_sweep_shape, lpm_release_workspace

integer(c_int), parameter :: LPM_MODE_FP64 = 0
integer(c_int), parameter :: LPM_MODE_FP32C = 1
integer(c_int), parameter :: LPM_PSE_K8_GEODESIC = 0
integer(c_int), parameter :: LPM_PSE_GAUSS_CHORD = 1
integer(c_int), parameter :: LPM_PSE_K8_CHORD = 2
integer(c_int), parameter :: LPM_GEOMETRY_PLANE = 0
integer(c_int), parameter :: LPM_GEOMETRY_SPHERE = 1

interface
	integer(c_int) function lpm_bve_velocity(n, x, y, z, zeta, area, active, radius, i_begin, i_end, &
			u, v, w, mode) bind(C, name="lpm_bve_velocity")
		import :: c_int, c_int32_t, c_int64_t, c_double
		integer(c_int64_t), value :: n
		real(c_double), intent(in) :: x(*), y(*), z(*), zeta(*), area(*)
		integer(c_int32_t), intent(in) :: active(*)
		real(c_double), value :: radius
		integer(c_int64_t), value :: i_begin, i_end
		real(c_double), intent(inout) :: u(*), v(*), w(*)
		integer(c_int), value :: mode
	end function

	integer(c_int) function lpm_bve_set_velocity_from_vorticity(n, x, y, z, zeta, area, active, radius, &
			i_begin, i_end, u, v, w, mode) bind(C, name="lpm_bve_set_velocity_from_vorticity")
		import :: c_int, c_int32_t, c_int64_t, c_double
		integer(c_int64_t), value :: n
		real(c_double), intent(in) :: x(*), y(*), z(*), zeta(*), area(*)
		integer(c_int32_t), intent(in) :: active(*)
		real(c_double), value :: radius
		integer(c_int64_t), value :: i_begin, i_end
		real(c_double), intent(inout) :: u(*), v(*), w(*)
		integer(c_int), value :: mode
	end function

	integer(c_int) function lpm_plane_velocity(n, x, y, omega, area, active, delta, i_begin, i_end, &
			u, v, mode) bind(C, name="lpm_plane_velocity")
		import :: c_int, c_int32_t, c_int64_t, c_double
		integer(c_int64_t), value :: n
		real(c_double), intent(in) :: x(*), y(*), omega(*), area(*)
		integer(c_int32_t), intent(in) :: active(*)
		real(c_double), value :: delta
		integer(c_int64_t), value :: i_begin, i_end
		real(c_double), intent(inout) :: u(*), v(*)
		integer(c_int), value :: mode
	end function

	integer(c_int) function lpm_pse_sphere_laplacian(n, x, y, z, f, area, active, eps, radius, kernel, &
			i_begin, i_end, lap, mode) bind(C, name="lpm_pse_sphere_laplacian")
		import :: c_int, c_int32_t, c_int64_t, c_double
		integer(c_int64_t), value :: n
		real(c_double), intent(in) :: x(*), y(*), z(*), f(*), area(*)
		integer(c_int32_t), intent(in) :: active(*)
		real(c_double), value :: eps, radius
		integer(c_int), value :: kernel
		integer(c_int64_t), value :: i_begin, i_end
		real(c_double), intent(inout) :: lap(*)
		integer(c_int), value :: mode
	end function

	integer(c_int) function lpm_pse_plane_laplacian(n, x, y, f, area, active, eps, kernel, &
			i_begin, i_end, lap, mode) bind(C, name="lpm_pse_plane_laplacian")
		import :: c_int, c_int32_t, c_int64_t, c_double
		integer(c_int64_t), value :: n
		real(c_double), intent(in) :: x(*), y(*), f(*), area(*)
		integer(c_int32_t), intent(in) :: active(*)
		real(c_double), value :: eps
		integer(c_int), value :: kernel
		integer(c_int64_t), value :: i_begin, i_end
		real(c_double), intent(inout) :: lap(*)
		integer(c_int), value :: mode
	end function

	integer(c_int) function lpm_bve_stream_functions(n, x, y, z, relvort, absvort, area, active, radius, &
			i_begin, i_end, psi_rel, psi_abs, mode) bind(C, name="lpm_bve_stream_functions")
		import :: c_int, c_int32_t, c_int64_t, c_double
		integer(c_int64_t), value :: n
		real(c_double), intent(in) :: x(*), y(*), z(*), relvort(*), absvort(*), area(*)
		integer(c_int32_t), intent(in) :: active(*)
		real(c_double), value :: radius
		integer(c_int64_t), value :: i_begin, i_end
		real(c_double), intent(inout) :: psi_rel(*), psi_abs(*)
		integer(c_int), value :: mode
	end function

	integer(c_int) function lpm_plane_stream_function(n, x, y, omega, area, active, i_begin, i_end, &
			psi, mode) bind(C, name="lpm_plane_stream_function")
		import :: c_int, c_int32_t, c_int64_t, c_double
		integer(c_int64_t), value :: n
		real(c_double), intent(in) :: x(*), y(*), omega(*), area(*)
		integer(c_int32_t), intent(in) :: active(*)
		integer(c_int64_t), value :: i_begin, i_end
		real(c_double), intent(inout) :: psi(*)
		integer(c_int), value :: mode
	end function

	integer(c_int) function lpm_pse_sphere_gradient(n, x, y, z, f, area, active, eps, radius, &
			i_begin, i_end, gx, gy, gz, mode) bind(C, name="lpm_pse_sphere_gradient")
		import :: c_int, c_int32_t, c_int64_t, c_double
		integer(c_int64_t), value :: n
		real(c_double), intent(in) :: x(*), y(*), z(*), f(*), area(*)
		integer(c_int32_t), intent(in) :: active(*)
		real(c_double), value :: eps, radius
		integer(c_int64_t), value :: i_begin, i_end
		real(c_double), intent(inout) :: gx(*), gy(*), gz(*)
		integer(c_int), value :: mode
	end function

	integer(c_int) function lpm_pse_sphere_divergence(n, x, y, z, vx, vy, vz, area, active, eps, radius, &
			i_begin, i_end, div, mode) bind(C, name="lpm_pse_sphere_divergence")
		import :: c_int, c_int32_t, c_int64_t, c_double
		integer(c_int64_t), value :: n
		real(c_double), intent(in) :: x(*), y(*), z(*), vx(*), vy(*), vz(*), area(*)
		integer(c_int32_t), intent(in) :: active(*)
		real(c_double), value :: eps, radius
		integer(c_int64_t), value :: i_begin, i_end
		real(c_double), intent(inout) :: div(*)
		integer(c_int), value :: mode
	end function

	integer(c_int) function lpm_pse_plane_gradient(n, x, y, f, area, active, eps, i_begin, i_end, gx, gy, &
			mode) bind(C, name="lpm_pse_plane_gradient")
		import :: c_int, c_int32_t, c_int64_t, c_double
		integer(c_int64_t), value :: n
		real(c_double), intent(in) :: x(*), y(*), f(*), area(*)
		integer(c_int32_t), intent(in) :: active(*)
		real(c_double), value :: eps
		integer(c_int64_t), value :: i_begin, i_end
		real(c_double), intent(inout) :: gx(*), gy(*)
		integer(c_int), value :: mode
	end function

	integer(c_int) function lpm_pse_plane_second_partials(n, x, y, gx, gy, area, active, eps, i_begin, i_end, &
			dxx, dxy, dyy, mode) bind(C, name="lpm_pse_plane_second_partials")
		import :: c_int, c_int32_t, c_int64_t, c_double
		integer(c_int64_t), value :: n
		real(c_double), intent(in) :: x(*), y(*), gx(*), gy(*), area(*)
		integer(c_int32_t), intent(in) :: active(*)
		real(c_double), value :: eps
		integer(c_int64_t), value :: i_begin, i_end
		real(c_double), intent(inout) :: dxx(*), dxy(*), dyy(*)
		integer(c_int), value :: mode
	end function

	integer(c_int) function lpm_pse_plane_double_dot(n, x, y, u, v, area, active, eps, i_begin, i_end, ddot, &
			mode) bind(C, name="lpm_pse_plane_double_dot")
		import :: c_int, c_int32_t, c_int64_t, c_double
		integer(c_int64_t), value :: n
		real(c_double), intent(in) :: x(*), y(*), u(*), v(*), area(*)
		integer(c_int32_t), intent(in) :: active(*)
		real(c_double), value :: eps
		integer(c_int64_t), value :: i_begin, i_end
		real(c_double), intent(inout) :: ddot(*)
		integer(c_int), value :: mode
	end function

	integer(c_int) function lpm_pse_sphere_double_dot(n, x, y, z, u, v, w, area, active, eps, radius, &
			i_begin, i_end, ddot, mode) bind(C, name="lpm_pse_sphere_double_dot")
		import :: c_int, c_int32_t, c_int64_t, c_double
		integer(c_int64_t), value :: n
		real(c_double), intent(in) :: x(*), y(*), z(*), u(*), v(*), w(*), area(*)
		integer(c_int32_t), intent(in) :: active(*)
		real(c_double), value :: eps, radius
		integer(c_int64_t), value :: i_begin, i_end
		real(c_double), intent(inout) :: ddot(*)
		integer(c_int), value :: mode
	end function

	integer(c_int) function lpm_pse_interpolate_scalar(n, x, y, z, f, area, active, eps, radius, geometry, &
			m, qx, qy, qz, out, mode) bind(C, name="lpm_pse_interpolate_scalar")
		import :: c_int, c_int32_t, c_int64_t, c_double
		integer(c_int64_t), value :: n
		real(c_double), intent(in) :: x(*), y(*), z(*), f(*), area(*)
		integer(c_int32_t), intent(in) :: active(*)
		real(c_double), value :: eps, radius
		integer(c_int), value :: geometry
		integer(c_int64_t), value :: m
		real(c_double), intent(in) :: qx(*), qy(*), qz(*)
		real(c_double), intent(inout) :: out(*)
		integer(c_int), value :: mode
	end function

	integer(c_int) function lpm_swe_plane_rhs_integrals(n, x, y, vort, div, surf_height, area, active, eps, &
			i_begin, i_end, u, v, double_dot, lap_surf, mode) bind(C, name="lpm_swe_plane_rhs_integrals")
		import :: c_int, c_int32_t, c_int64_t, c_double
		integer(c_int64_t), value :: n
		real(c_double), intent(in) :: x(*), y(*), vort(*), div(*), surf_height(*), area(*)
		integer(c_int32_t), intent(in) :: active(*)
		real(c_double), value :: eps
		integer(c_int64_t), value :: i_begin, i_end
		real(c_double), intent(inout) :: u(*), v(*), double_dot(*), lap_surf(*)
		integer(c_int), value :: mode
	end function

	integer(c_int) function lpm_swe_sphere_rhs_integrals(n, x, y, z, relvort, div, surf_height, area, active, &
			radius, sphere_radius, eps, i_begin, i_end, u, v, w, double_dot, lap_surf, mode) &
			bind(C, name="lpm_swe_sphere_rhs_integrals")
		import :: c_int, c_int32_t, c_int64_t, c_double
		integer(c_int64_t), value :: n
		real(c_double), intent(in) :: x(*), y(*), z(*), relvort(*), div(*), surf_height(*), area(*)
		integer(c_int32_t), intent(in) :: active(*)
		real(c_double), value :: radius, sphere_radius, eps
		integer(c_int64_t), value :: i_begin, i_end
		real(c_double), intent(inout) :: u(*), v(*), w(*), double_dot(*), lap_surf(*)
		integer(c_int), value :: mode
	end function

	integer(c_int) function lpm_plane_solver_remesh(solver, n, x, y, omega, area, active, u, v) &
			bind(C, name="lpm_plane_solver_remesh")
		import :: c_int, c_int32_t, c_int64_t, c_double, c_ptr
		type(c_ptr), value :: solver
		integer(c_int64_t), value :: n
		real(c_double), intent(in) :: x(*), y(*), omega(*), area(*)
		integer(c_int32_t), intent(in) :: active(*)
		type(c_ptr), value :: u, v
	end function

	integer(c_int) function lpm_bve_solver_remesh(solver, n, x, y, z, relvort, area, active, u, v, w) &
			bind(C, name="lpm_bve_solver_remesh")
		import :: c_int, c_int32_t, c_int64_t, c_double, c_ptr
		type(c_ptr), value :: solver
		integer(c_int64_t), value :: n
		real(c_double), intent(in) :: x(*), y(*), z(*), relvort(*), area(*)
		integer(c_int32_t), intent(in) :: active(*)
		type(c_ptr), value :: u, v, w
	end function

	integer(c_int) function lpm_beta_plane_velocity(n, x, y, zeta, area, active, i_begin, i_end, u, v, mode) &
			bind(C, name="lpm_beta_plane_velocity")
		import :: c_int, c_int32_t, c_int64_t, c_double
		integer(c_int64_t), value :: n
		real(c_double), intent(in) :: x(*), y(*), zeta(*), area(*)
		integer(c_int32_t), intent(in) :: active(*)
		integer(c_int64_t), value :: i_begin, i_end
		real(c_double), intent(inout) :: u(*), v(*)
		integer(c_int), value :: mode
	end function

	integer(c_int) function lpm_beta_plane_stream_functions(n, x, y, relvort, absvort, area, active, i_begin, &
			i_end, psi_rel, psi_abs, mode) bind(C, name="lpm_beta_plane_stream_functions")
		import :: c_int, c_int32_t, c_int64_t, c_double
		integer(c_int64_t), value :: n
		real(c_double), intent(in) :: x(*), y(*), relvort(*), absvort(*), area(*)
		integer(c_int32_t), intent(in) :: active(*)
		integer(c_int64_t), value :: i_begin, i_end
		real(c_double), intent(inout) :: psi_rel(*), psi_abs(*)
		integer(c_int), value :: mode
	end function

	type(c_ptr) function lpm_last_error_string() bind(C, name="lpm_last_error_string")
		import :: c_ptr
	end function

	! ---- device-resident BVESolver (timestepPrivate, src/SphereBVESolver.f90:219-353).
	! u, v, w may be c_null_ptr (then the initial velocity is computed on the device);
	! otherwise pass c_loc of the arrays.
	integer(c_int) function lpm_bve_solver_create(solver, n, x, y, z, relvort, area, active, u, v, w, &
			radius, rotation_rate, mode) bind(C, name="lpm_bve_solver_create")
		import :: c_int, c_int32_t, c_int64_t, c_double, c_ptr
		type(c_ptr), intent(out) :: solver
		integer(c_int64_t), value :: n
		real(c_double), intent(in) :: x(*), y(*), z(*), relvort(*), area(*)
		integer(c_int32_t), intent(in) :: active(*)
		type(c_ptr), value :: u, v, w
		real(c_double), value :: radius, rotation_rate
		integer(c_int), value :: mode
	end function

	integer(c_int) function lpm_bve_timestep(solver, dt, n_steps, renormalize) bind(C, name="lpm_bve_timestep")
		import :: c_int, c_double, c_ptr
		type(c_ptr), value :: solver
		real(c_double), value :: dt
		integer(c_int), value :: n_steps, renormalize
	end function

	integer(c_int) function lpm_bve_get_state(solver, x, y, z, relvort, u, v, w) bind(C, name="lpm_bve_get_state")
		import :: c_int, c_double, c_ptr
		type(c_ptr), value :: solver
		real(c_double), intent(out) :: x(*), y(*), z(*), relvort(*), u(*), v(*), w(*)
	end function

	integer(c_int) function lpm_bve_set_state(solver, x, y, z, relvort, u, v, w) bind(C, name="lpm_bve_set_state")
		import :: c_int, c_double, c_ptr
		type(c_ptr), value :: solver
		real(c_double), intent(in) :: x(*), y(*), z(*), relvort(*), u(*), v(*), w(*)
	end function

	integer(c_int) function lpm_bve_diagnostics(solver, kinetic_energy, enstrophy, circulation) &
			bind(C, name="lpm_bve_diagnostics")
		import :: c_int, c_double, c_ptr
		type(c_ptr), value :: solver
		real(c_double), intent(out) :: kinetic_energy, enstrophy, circulation
	end function

	! SetStreamFunctionsOnMesh at the solver's state (the call at src/SphereBVESolver.f90:352);
	! absvort may be c_null_ptr (then zeta + 2 Omega z / a of the state is used).
	integer(c_int) function lpm_bve_solver_stream_functions(solver, absvort, psi_rel, psi_abs) &
			bind(C, name="lpm_bve_solver_stream_functions")
		import :: c_int, c_double, c_ptr
		type(c_ptr), value :: solver, absvort
		real(c_double), intent(out) :: psi_rel(*), psi_abs(*)
	end function

	integer(c_int) function lpm_bve_solver_destroy(solver) bind(C, name="lpm_bve_solver_destroy")
		import :: c_int, c_ptr
		type(c_ptr), value :: solver
	end function

	! ---- device-resident PlaneSolver (timestepPrivate, src/PlaneIncompressibleSolver.f90:171-259)
	integer(c_int) function lpm_plane_solver_create(solver, n, x, y, omega, area, active, u, v, delta, mode) &
			bind(C, name="lpm_plane_solver_create")
		import :: c_int, c_int32_t, c_int64_t, c_double, c_ptr
		type(c_ptr), intent(out) :: solver
		integer(c_int64_t), value :: n
		real(c_double), intent(in) :: x(*), y(*), omega(*), area(*)
		integer(c_int32_t), intent(in) :: active(*)
		type(c_ptr), value :: u, v
		real(c_double), value :: delta
		integer(c_int), value :: mode
	end function

	integer(c_int) function lpm_plane_timestep(solver, dt, n_steps) bind(C, name="lpm_plane_timestep")
		import :: c_int, c_double, c_ptr
		type(c_ptr), value :: solver
		real(c_double), value :: dt
		integer(c_int), value :: n_steps
	end function

	integer(c_int) function lpm_plane_get_state(solver, x, y, u, v) bind(C, name="lpm_plane_get_state")
		import :: c_int, c_double, c_ptr
		type(c_ptr), value :: solver
		real(c_double), intent(out) :: x(*), y(*), u(*), v(*)
	end function

	integer(c_int) function lpm_plane_diagnostics(solver, kinetic_energy, enstrophy, circulation) &
			bind(C, name="lpm_plane_diagnostics")
		import :: c_int, c_double, c_ptr
		type(c_ptr), value :: solver
		real(c_double), intent(out) :: kinetic_energy, enstrophy, circulation
	end function

	integer(c_int) function lpm_plane_solver_destroy(solver) bind(C, name="lpm_plane_solver_destroy")
		import :: c_int, c_ptr
		type(c_ptr), value :: solver
	end function

	! ---- many BVE instances advanced together (instance k owns offsets(k+1) .. offsets(k+2)-1,
	!      0-based, of the concatenated arrays; radius and rotation_rate per instance)
	integer(c_int) function lpm_ensemble_create(ens, n_instances, offsets, x, y, z, relvort, area, active, &
			radius, rotation_rate, mode) bind(C, name="lpm_ensemble_create")
		import :: c_int, c_int32_t, c_int64_t, c_double, c_ptr
		type(c_ptr), intent(out) :: ens
		integer(c_int), value :: n_instances
		integer(c_int64_t), intent(in) :: offsets(*)
		real(c_double), intent(in) :: x(*), y(*), z(*), relvort(*), area(*), radius(*), rotation_rate(*)
		integer(c_int32_t), intent(in) :: active(*)
		integer(c_int), value :: mode
	end function

	integer(c_int) function lpm_ensemble_timestep(ens, dt, n_steps, renormalize) bind(C, name="lpm_ensemble_timestep")
		import :: c_int, c_double, c_ptr
		type(c_ptr), value :: ens
		real(c_double), value :: dt
		integer(c_int), value :: n_steps, renormalize
	end function

	integer(c_int) function lpm_ensemble_velocity(ens) bind(C, name="lpm_ensemble_velocity")
		import :: c_int, c_ptr
		type(c_ptr), value :: ens
	end function

	integer(c_int) function lpm_ensemble_get_state(ens, x, y, z, relvort, u, v, w) &
			bind(C, name="lpm_ensemble_get_state")
		import :: c_int, c_double, c_ptr
		type(c_ptr), value :: ens
		real(c_double), intent(out) :: x(*), y(*), z(*), relvort(*), u(*), v(*), w(*)
	end function

	integer(c_int) function lpm_ensemble_destroy(ens) bind(C, name="lpm_ensemble_destroy")
		import :: c_int, c_ptr
		type(c_ptr), value :: ens
	end function

	integer(c_int) function lpm_ensemble_sweep_shape(ens, threads, targetsPerThread, ctasPerSM, itemsPerSlot) &
			bind(C, name="lpm_ensemble_sweep_shape")
		import :: c_int, c_ptr
		type(c_ptr), value :: ens
		integer(c_int), intent(out) :: threads, targetsPerThread, ctasPerSM, itemsPerSlot
	end function

	! ---- workspace
	integer(c_int) function lpm_release_workspace() bind(C, name="lpm_release_workspace")
		import :: c_int
	end function

	! ---- timing and version
	integer(c_int) function lpm_bve_kernel_timing(solver, total_ms, launches) bind(C, name="lpm_bve_kernel_timing")
		import :: c_int, c_int64_t, c_double, c_ptr
		type(c_ptr), value :: solver
		real(c_double), intent(out) :: total_ms
		integer(c_int64_t), intent(out) :: launches
	end function

	integer(c_int) function lpm_bve_solver_set_timing(solver, enable) bind(C, name="lpm_bve_solver_set_timing")
		import :: c_int, c_ptr
		type(c_ptr), value :: solver
		integer(c_int), value :: enable
	end function

	type(c_ptr) function lpm_version() bind(C, name="lpm_version")
		import :: c_ptr
	end function
end interface

contains

!> @brief logical(klog) mask -> int32 0/1 array (done once per solver New; the mask only
!> changes at a remesh, when the solver is rebuilt).
subroutine GpuMask(mask32, mask)
	integer(c_int32_t), allocatable, intent(inout) :: mask32(:)
	logical(klog), intent(in) :: mask(:)
	if (allocated(mask32)) deallocate(mask32)
	allocate(mask32(size(mask)))
	mask32 = merge(1_c_int32_t, 0_c_int32_t, mask)
end subroutine

!> @brief Maps a non-zero status to a Logger ERROR message (which clears testPass).
subroutine GpuStatusCheck(rc, aLog, where)
	integer(c_int), intent(in) :: rc
	type(Logger), intent(inout) :: aLog
	character(len=*), intent(in) :: where
	character(kind=c_char), pointer :: msg(:)
	character(len=512) :: text
	integer :: i
	if (rc == 0) return
	call c_f_pointer(lpm_last_error_string(), msg, [512])
	text = ' '
	do i = 1, 512
		if (msg(i) == c_null_char) exit
		text(i:i) = msg(i)
	enddo
	call LogMessage(aLog, ERROR_LOGGING_LEVEL, where//" liblpm_gpu ERROR : ", trim(text))
end subroutine

!> @brief Body of BVESphereVelocity (src/SphereBVESolver.f90:377-430) on the GPU: the same
!> arguments, with the int32 mask and the rank's block instead of the MPISetup object.
subroutine GpuBVESphereVelocity(u, v, w, x, y, z, relVortIn, areaIn, sphereRadius, mask32, &
		indexStart, indexEnd, mode, aLog)
	real(kreal), dimension(:), intent(inout) :: u, v, w
	real(kreal), dimension(:), intent(in) :: x, y, z, relVortIn, areaIn
	real(kreal), intent(in) :: sphereRadius
	integer(c_int32_t), dimension(:), intent(in) :: mask32
	integer(kint), intent(in) :: indexStart, indexEnd
	integer(c_int), intent(in) :: mode
	type(Logger), intent(inout) :: aLog
	integer(c_int) :: rc
	rc = lpm_bve_velocity(int(size(x), c_int64_t), x, y, z, relVortIn, areaIn, mask32, sphereRadius, &
		int(indexStart, c_int64_t), int(indexEnd, c_int64_t), u, v, w, mode)
	call GpuStatusCheck(rc, aLog, "BVESphereVelocity")
end subroutine

!> @brief Body of planarIncompressibleVelocity (src/PlaneIncompressibleSolver.f90:278-316).
subroutine GpuPlanarVelocity(u, v, x, y, vortIn, areaIn, mask32, delta, indexStart, indexEnd, mode, aLog)
	real(kreal), dimension(:), intent(inout) :: u, v
	real(kreal), dimension(:), intent(in) :: x, y, vortIn, areaIn
	integer(c_int32_t), dimension(:), intent(in) :: mask32
	real(kreal), intent(in) :: delta
	integer(kint), intent(in) :: indexStart, indexEnd
	integer(c_int), intent(in) :: mode
	type(Logger), intent(inout) :: aLog
	integer(c_int) :: rc
	rc = lpm_plane_velocity(int(size(x), c_int64_t), x, y, vortIn, areaIn, mask32, delta, &
		int(indexStart, c_int64_t), int(indexEnd, c_int64_t), u, v, mode)
	call GpuStatusCheck(rc, aLog, "planarIncompressibleVelocity")
end subroutine

!> @brief Body of PSESphereLaplacianAtParticles (src/PSEDirectSum.f90:502-535), including its
!> final multiplication by 1/eps**2.
subroutine GpuPSESphereLaplacian(lap, x, y, z, f, area, mask32, eps, radius, indexStart, indexEnd, mode, aLog)
	real(kreal), dimension(:), intent(inout) :: lap
	real(kreal), dimension(:), intent(in) :: x, y, z, f, area
	integer(c_int32_t), dimension(:), intent(in) :: mask32
	real(kreal), intent(in) :: eps, radius
	integer(kint), intent(in) :: indexStart, indexEnd
	integer(c_int), intent(in) :: mode
	type(Logger), intent(inout) :: aLog
	integer(c_int) :: rc
	rc = lpm_pse_sphere_laplacian(int(size(x), c_int64_t), x, y, z, f, area, mask32, eps, radius, &
		LPM_PSE_K8_GEODESIC, int(indexStart, c_int64_t), int(indexEnd, c_int64_t), lap, mode)
	call GpuStatusCheck(rc, aLog, "PSESphereLaplacianAtParticles")
end subroutine

end module
