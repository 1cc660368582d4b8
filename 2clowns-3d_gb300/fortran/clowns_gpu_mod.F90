!%%%%%%%%%%%%%%%%%%%%% FILE: clowns_gpu_mod.F90 %%%%%%%%%%%%%%%%%%%%%%%%%%%%%%%%
! ISO_C_BINDING interface to libclowns_gpu.so (the GB300 pressure solve): one
! bind(C) interface for every function of include/clowns_gpu.h.
!
! Two ways to use it from the model:
!
!  1. Link-level drop-in: link libclowns_gpu.so instead of pcgpme_para.o (and
!     pcgpme_2DH.o).  The library exports pcgpme_ and pcgpme_will_ (ifort's
!     names for PCGPME and PCGPME_WILL), so cal_poisson_equation and
!     disp_adjust keep their calls unchanged.
!
!  2. Explicit calls through the interfaces below, e.g. the device-resident
!     entry points when the module arrays are kept on the GPU by the host code,
!     or the pcgpme_via_gpu / pcgpme_will_via_gpu wrappers in a source swap.
!
! Conventions.  Host arrays cross as assumed-size dummies (by reference);
! device addresses (the *_dev functions, obtained e.g. from cudaMalloc through
! a CUDA Fortran or C helper) and the stream cross as type(c_ptr), value.
! The reference's routines without arguments (set_nflag, init_matrix,
! cal_err_of_continuity, cal_matrix_element, estimate_velocity2) take the
! module arrays of `arrays` explicitly: Fortran module descriptors are
! compiler-specific, so only raw arrays cross the boundary, with the lower
! bounds listed at the top of include/clowns_gpu.h.  The derived type cellflag
! crosses as two integer arrays nff(:)%f and nff(:)%b.  Every function that
! returns integer(c_int) returns 0 or a negative CLOWNS_ERR_* code, described
! by clowns_error_message().
!
! This file is not compiled in this repository (no Fortran compiler is
! available where it was written); a CPU test checks that it declares every
! function of the C header with the header's argument count.
module clowns_gpu
    use iso_c_binding
    implicit none

    integer(c_int), parameter :: CLOWNS_OK = 0, CLOWNS_ERR_CUDA = -1, CLOWNS_ERR_ARG = -2
    integer(c_int), parameter :: CLOWNS_ERR_WORKSPACE = -3, CLOWNS_ERR_NOCONV = -4, CLOWNS_ERR_LIMIT = -5
    integer(c_int), parameter :: CLOWNS_PREC_FP64 = 0, CLOWNS_PREC_MIXED = 1

    type, bind(C) :: clowns_solve_info
        real(c_double) :: eps, bn
        integer(c_int) :: iter, ier, reason, outer
    end type clowns_solve_info

    ! one system of an ensemble (device addresses)
    type, bind(C) :: clowns_member
        type(c_ptr) :: al, ll, d, b, x
        integer(c_int) :: na, n, nl, pad
    end type clowns_member

    interface
        ! ---- errors and version ------------------------------------------------
        type(c_ptr) function clowns_last_error() bind(C, name="clowns_last_error")
            import :: c_ptr
        end function clowns_last_error

        integer(c_int) function clowns_version() bind(C, name="clowns_version")
            import :: c_int
        end function clowns_version

        ! ---- PCGPME drop-in with host arrays (same arguments, by reference) -------
        subroutine pcgpme_gpu(al, nl, na, ll, d, n, n2, b, x, eps, parm, iter, ier) &
                bind(C, name="pcgpme_gpu")
            import :: c_double, c_int
            real(c_double), intent(inout) :: al(*), d(*), b(*), x(*), eps(2)
            integer(c_int), intent(in) :: nl, na, n, n2
            integer(c_int), intent(inout) :: ll(*), iter
            real(c_double), intent(in) :: parm
            integer(c_int), intent(out) :: ier
        end subroutine pcgpme_gpu

        ! the same function under ifort's name for PCGPME (link-level drop-in)
        subroutine pcgpme_link_alias(al, nl, na, ll, d, n, n2, b, x, eps, parm, iter, ier) &
                bind(C, name="pcgpme_")
            import :: c_double, c_int
            real(c_double), intent(inout) :: al(*), d(*), b(*), x(*), eps(2)
            integer(c_int), intent(in) :: nl, na, n, n2
            integer(c_int), intent(inout) :: ll(*), iter
            real(c_double), intent(in) :: parm
            integer(c_int), intent(out) :: ier
        end subroutine pcgpme_link_alias

        ! ---- device-resident PCGPME ------------------------------------------------
        integer(c_size_t) function clowns_pcgpme_workspace_bytes(n, nl) &
                bind(C, name="clowns_pcgpme_workspace_bytes")
            import :: c_int, c_size_t
            integer(c_int), value :: n, nl
        end function clowns_pcgpme_workspace_bytes

        integer(c_int) function clowns_pcgpme_dev(al, nl, na, ll, d, n, b, x, eps, parm, iter, &
                work, work_bytes, stream, info) bind(C, name="clowns_pcgpme_dev")
            import :: c_int, c_double, c_ptr, c_size_t, clowns_solve_info
            type(c_ptr), value :: al, ll, d, b, x, work, stream
            integer(c_int), value :: nl, na, n, iter
            real(c_double), value :: eps, parm
            integer(c_size_t), value :: work_bytes
            type(clowns_solve_info), intent(out) :: info
        end function clowns_pcgpme_dev

        ! ---- mixed precision and batched ensembles --------------------------------
        integer(c_size_t) function clowns_pcgpme_mixed_workspace_bytes(n, nl) &
                bind(C, name="clowns_pcgpme_mixed_workspace_bytes")
            import :: c_int, c_size_t
            integer(c_int), value :: n, nl
        end function clowns_pcgpme_mixed_workspace_bytes

        integer(c_int) function clowns_pcgpme_mixed_dev(al, nl, na, ll, d, n, b, x, eps, parm, &
                inner_tol, inner_max, max_outer, work, work_bytes, stream, info) &
                bind(C, name="clowns_pcgpme_mixed_dev")
            import :: c_int, c_double, c_ptr, c_size_t, clowns_solve_info
            type(c_ptr), value :: al, ll, d, b, x, work, stream
            integer(c_int), value :: nl, na, n, inner_max, max_outer
            real(c_double), value :: eps, parm, inner_tol
            integer(c_size_t), value :: work_bytes
            type(clowns_solve_info), intent(out) :: info
        end function clowns_pcgpme_mixed_dev

        integer(c_size_t) function clowns_pcgpme_batched_workspace_bytes(m, n, precision) &
                bind(C, name="clowns_pcgpme_batched_workspace_bytes")
            import :: c_int, c_size_t
            integer(c_int), value :: m, precision
            integer(c_int), intent(in) :: n(*)
        end function clowns_pcgpme_batched_workspace_bytes

        integer(c_int) function clowns_pcgpme_batched_dev(m, members, precision, eps, parm, iter, &
                inner_tol, inner_max, max_outer, work, work_bytes, stream, infos) &
                bind(C, name="clowns_pcgpme_batched_dev")
            import :: c_int, c_double, c_ptr, c_size_t, clowns_member, clowns_solve_info
            integer(c_int), value :: m, precision, iter, inner_max, max_outer
            type(clowns_member), intent(in) :: members(*)
            real(c_double), value :: eps, parm, inner_tol
            type(c_ptr), value :: work, stream
            integer(c_size_t), value :: work_bytes
            type(clowns_solve_info), intent(out) :: infos(*)
        end function clowns_pcgpme_batched_dev

        integer(c_int) function clowns_tuned_shape(m, n, precision, mode, block, grid, regs, fused) &
                bind(C, name="clowns_tuned_shape")
            import :: c_int
            integer(c_int), value :: m, precision
            integer(c_int), intent(in) :: n(*)
            integer(c_int), intent(out) :: mode, block, grid, regs, fused
        end function clowns_tuned_shape

        integer(c_int) function clowns_test_arm_wait_timeout(polls, absent_block) &
                bind(C, name="clowns_test_arm_wait_timeout")
            import :: c_int, c_long
            integer(c_long), value :: polls
            integer(c_int), value :: absent_block
        end function clowns_test_arm_wait_timeout

        integer(c_long) function clowns_last_kernel_launches() bind(C, name="clowns_last_kernel_launches")
            import :: c_long
        end function clowns_last_kernel_launches

        ! measured FP64 fused multiply-add rate of the device (lane operations per second)
        integer(c_int) function clowns_fp64_fma_rate(fma_per_s, stream) bind(C, name="clowns_fp64_fma_rate")
            import :: c_int, c_double, c_ptr
            real(c_double), intent(out) :: fma_per_s
            type(c_ptr), value :: stream
        end function clowns_fp64_fma_rate

        ! ---- PCGPME_WILL (2DH dispersion solve) --------------------------------------
        ! host arrays; B in: RHS, out: what the reference leaves in B
        integer(c_int) function pcgpme_will_gpu(al, nl, na, ll, d, n, n2, b, eps, parm, iter) &
                bind(C, name="pcgpme_will_gpu")
            import :: c_double, c_int
            real(c_double), intent(in) :: al(*), d(*), eps, parm
            integer(c_int), intent(in) :: nl, na, n, n2, iter, ll(*)
            real(c_double), intent(inout) :: b(*)
        end function pcgpme_will_gpu

        ! the same function under ifort's name for PCGPME_WILL (link-level drop-in)
        integer(c_int) function pcgpme_will_link_alias(al, nl, na, ll, d, n, n2, b, eps, parm, iter) &
                bind(C, name="pcgpme_will_")
            import :: c_double, c_int
            real(c_double), intent(in) :: al(*), d(*), eps, parm
            integer(c_int), intent(in) :: nl, na, n, n2, iter, ll(*)
            real(c_double), intent(inout) :: b(*)
        end function pcgpme_will_link_alias

        integer(c_size_t) function clowns_pcgpme_will_workspace_bytes(n, nl) &
                bind(C, name="clowns_pcgpme_will_workspace_bytes")
            import :: c_int, c_size_t
            integer(c_int), value :: n, nl
        end function clowns_pcgpme_will_workspace_bytes

        integer(c_int) function clowns_pcgpme_will_dev(al, nl, na, ll, d, n, b, eps, parm, iter, &
                work, work_bytes, stream, info) bind(C, name="clowns_pcgpme_will_dev")
            import :: c_int, c_double, c_ptr, c_size_t, clowns_solve_info
            type(c_ptr), value :: al, ll, d, b, work, stream
            integer(c_int), value :: nl, na, n, iter
            real(c_double), value :: eps, parm
            integer(c_size_t), value :: work_bytes
            type(clowns_solve_info), intent(out) :: info
        end function clowns_pcgpme_will_dev

        integer(c_size_t) function clowns_will_postprocess_workspace_bytes(n) &
                bind(C, name="clowns_will_postprocess_workspace_bytes")
            import :: c_int, c_size_t
            integer(c_int), value :: n
        end function clowns_will_postprocess_workspace_bytes

        integer(c_int) function clowns_will_postprocess_dev(x, r, ll, nl, na, n, b, x_out, work, &
                work_bytes, stream) bind(C, name="clowns_will_postprocess_dev")
            import :: c_int, c_ptr, c_size_t
            type(c_ptr), value :: x, r, ll, b, x_out, work, stream
            integer(c_int), value :: nl, na, n
            integer(c_size_t), value :: work_bytes
        end function clowns_will_postprocess_dev

        ! ---- building blocks of the solve (device arrays) ---------------------------
        integer(c_int) function clowns_pcgpme_setup_dev(al, nl, na, ll, d, n, b, parm, al_s, ll_s, &
                d_s, b_s, na_out, work, work_bytes, stream) bind(C, name="clowns_pcgpme_setup_dev")
            import :: c_int, c_double, c_ptr, c_size_t
            type(c_ptr), value :: al, ll, d, b, al_s, ll_s, d_s, b_s, work, stream
            integer(c_int), value :: nl, na, n, na_out
            real(c_double), value :: parm
            integer(c_size_t), value :: work_bytes
        end function clowns_pcgpme_setup_dev

        integer(c_int) function clowns_apply_pm_a_dev(al, nl, na, ll, d, n, parm, x, y, work, &
                work_bytes, stream) bind(C, name="clowns_apply_pm_a_dev")
            import :: c_int, c_double, c_ptr, c_size_t
            type(c_ptr), value :: al, ll, d, x, y, work, stream
            integer(c_int), value :: nl, na, n
            real(c_double), value :: parm
            integer(c_size_t), value :: work_bytes
        end function clowns_apply_pm_a_dev

        ! ---- set_nflag, init_matrix, rows + RHS, assembly, correction -------------
        integer(c_size_t) function clowns_set_nflag_workspace_bytes(dims, inne2) &
                bind(C, name="clowns_set_nflag_workspace_bytes")
            import :: c_int, c_size_t
            integer(c_int), intent(in) :: dims(6)
            integer(c_int), value :: inne2
        end function clowns_set_nflag_workspace_bytes

        ! set_nflag (nfd2015.F90:7-306); ifln, isfn, passes come back on the host
        integer(c_int) function clowns_set_nflag_dev(dims, inne, inne2, mx2, mn, in, jn, kn, nf, &
                nfb, f, fb, a, dx, objno, fln, ifln, sfn, isfn, passes, work, work_bytes, stream) &
                bind(C, name="clowns_set_nflag_dev")
            import :: c_int, c_ptr, c_size_t
            integer(c_int), intent(in) :: dims(6)
            integer(c_int), value :: inne, inne2, mx2
            type(c_ptr), value :: mn, in, jn, kn, nf, nfb, f, fb, a, dx, objno, fln, sfn, work, stream
            integer(c_int), intent(out) :: ifln, isfn, passes
            integer(c_size_t), value :: work_bytes
        end function clowns_set_nflag_dev

        ! the value init_matrix gives nl: 6 (3D), 4 (2DV), 0 (no matrix form)
        integer(c_int) function clowns_grid_nl(dims) bind(C, name="clowns_grid_nl")
            import :: c_int
            integer(c_int), intent(in) :: dims(6)
        end function clowns_grid_nl

        ! init_matrix (1sub-matrix.F90:3-66); mp is a device address
        integer(c_int) function clowns_init_matrix_dev(dims, inne, mx2, mn, in, jn, kn, nf, nfb, a, &
                fb, dx, mp, alu_c, ll_c, de_c, stream) bind(C, name="clowns_init_matrix_dev")
            import :: c_int, c_ptr
            integer(c_int), intent(in) :: dims(6)
            integer(c_int), value :: inne, mx2
            type(c_ptr), value :: mn, in, jn, kn, nf, nfb, a, fb, dx, mp, alu_c, ll_c, de_c, stream
        end function clowns_init_matrix_dev

        integer(c_size_t) function clowns_rows_rhs_workspace_bytes(ifln) &
                bind(C, name="clowns_rows_rhs_workspace_bytes")
            import :: c_int, c_size_t
            integer(c_int), value :: ifln
        end function clowns_rows_rhs_workspace_bytes

        ! cal_err_of_continuity at ik == 0 (1sub-momentum.F90:235-360); mnoe and
        ! dmax come back on the host
        integer(c_int) function clowns_rows_rhs_dev(dims, inne2, mx2, mn, in, jn, kn, nf, nfb, f, fb, &
                a, un, dx, mp, dt, ifln, fln, mm2, mno, mno2mn, b, xe, de, mnoe, dmax, work, &
                work_bytes, stream) bind(C, name="clowns_rows_rhs_dev")
            import :: c_int, c_double, c_ptr, c_size_t
            integer(c_int), intent(in) :: dims(6)
            integer(c_int), value :: inne2, mx2, ifln, mm2
            type(c_ptr), value :: mn, in, jn, kn, nf, nfb, f, fb, a, un, dx, mp, fln
            type(c_ptr), value :: mno, mno2mn, b, xe, de, work, stream
            real(c_double), value :: dt
            integer(c_int), intent(out) :: mnoe
            real(c_double), intent(out) :: dmax
            integer(c_size_t), value :: work_bytes
        end function clowns_rows_rhs_dev

        ! cal_matrix_element (1sub-momentum.F90:465-551)
        integer(c_int) function clowns_assemble_dev(dims, inne, inne2, mx2, in, jn, kn, nf, nfb, &
                x, dx, sp, ifln, fln, mno, alu_c, ll_c, de_c, mm2, alu, llu, de, err_cell, stream) &
                bind(C, name="clowns_assemble_dev")
            import :: c_int, c_ptr
            integer(c_int), intent(in) :: dims(6)
            integer(c_int), value :: inne, inne2, mx2, ifln, mm2
            type(c_ptr), value :: in, jn, kn, nf, nfb, x, dx, sp, fln, mno, alu_c, ll_c, de_c
            type(c_ptr), value :: alu, llu, de, err_cell, stream
        end function clowns_assemble_dev

        ! p -= xe and estimate_velocity2 (1sub-momentum.F90:52-58, 590-651); xe0 = xe(0)
        integer(c_int) function clowns_correct_dev(dims, inne, mx2, mn, in, jn, kn, nf, nfb, a, dx, &
                dt, mnoe, mno2mn, mno, xe0, p, un, stream) bind(C, name="clowns_correct_dev")
            import :: c_int, c_double, c_ptr
            integer(c_int), intent(in) :: dims(6)
            integer(c_int), value :: inne, mx2, mnoe
            type(c_ptr), value :: mn, in, jn, kn, nf, nfb, a, dx, mno2mn, mno, xe0, p, un, stream
            real(c_double), value :: dt
        end function clowns_correct_dev

        ! ---- discrete adjoint ---------------------------------------------------------
        integer(c_int) function clowns_transpose_dev(n, na, nl, alu, llu, de, alt, llt, det, bad, &
                stream) bind(C, name="clowns_transpose_dev")
            import :: c_int, c_ptr
            integer(c_int), value :: n, na, nl
            type(c_ptr), value :: alu, llu, de, alt, llt, det, bad, stream
        end function clowns_transpose_dev

        integer(c_int) function clowns_face_grad_dev(dims, inne, inne2, ifln, fln, in, jn, kn, nf, &
                mno, alu_c, ll_c, a, x, lambda, grad, stream) bind(C, name="clowns_face_grad_dev")
            import :: c_int, c_ptr
            integer(c_int), intent(in) :: dims(6)
            integer(c_int), value :: inne, inne2, ifln
            type(c_ptr), value :: fln, in, jn, kn, nf, mno, alu_c, ll_c, a, x, lambda, grad, stream
        end function clowns_face_grad_dev

        ! ---- allocation-free FP64 solve (n <= 32768) ------------------------------------
        integer(c_int) function clowns_pcgpme_static_dev(al, nl, na, ll, d, n, b, x, eps, parm, &
                iter, stream, info) bind(C, name="clowns_pcgpme_static_dev")
            import :: c_int, c_double, c_ptr, clowns_solve_info
            type(c_ptr), value :: al, ll, d, b, x, stream
            integer(c_int), value :: nl, na, n, iter
            real(c_double), value :: eps, parm
            type(clowns_solve_info), intent(out) :: info
        end function clowns_pcgpme_static_dev

        ! ---- the ik loop with the domain's arrays in HBM (host arrays in and out) ----
        integer(c_int) function clowns_session_create(s, dims, inne, inne2, mx2, mn, in, jn, kn, x, &
                dx, objno) bind(C, name="clowns_session_create")
            import :: c_int, c_double, c_ptr
            type(c_ptr), intent(out) :: s
            integer(c_int), intent(in) :: dims(6), mn(*), in(*), jn(*), kn(*), objno(*)
            integer(c_int), value :: inne, inne2, mx2
            real(c_double), intent(in) :: x(*), dx(*)
        end function clowns_session_create

        integer(c_int) function clowns_session_set_fields(s, nf, nfb, f, fb, a, un, sp, p) &
                bind(C, name="clowns_session_set_fields")
            import :: c_int, c_double, c_ptr
            type(c_ptr), value :: s
            integer(c_int), intent(in) :: nf(*), nfb(*)
            real(c_double), intent(in) :: f(*), fb(*), a(*), un(*), sp(*), p(*)
        end function clowns_session_set_fields

        integer(c_int) function clowns_session_classify(s, ifln, isfn) bind(C, name="clowns_session_classify")
            import :: c_int, c_ptr
            type(c_ptr), value :: s
            integer(c_int), intent(out) :: ifln, isfn
        end function clowns_session_classify

        integer(c_int) function clowns_session_pressure_loop(s, dt, d0, eps0, precision, ik, dmax, &
                iter, err, icon) bind(C, name="clowns_session_pressure_loop")
            import :: c_int, c_double, c_ptr
            type(c_ptr), value :: s
            real(c_double), value :: dt, d0, eps0
            integer(c_int), value :: precision
            integer(c_int), intent(out) :: ik, iter, icon
            real(c_double), intent(out) :: dmax, err
        end function clowns_session_pressure_loop

        integer(c_int) function clowns_session_get_fields(s, nf, nfb, f, p, un, mnoe) &
                bind(C, name="clowns_session_get_fields")
            import :: c_int, c_double, c_ptr
            type(c_ptr), value :: s
            integer(c_int), intent(out) :: nf(*), nfb(*), mnoe
            real(c_double), intent(out) :: f(*), p(*), un(*)
        end function clowns_session_get_fields

        integer(c_int) function clowns_session_destroy(s) bind(C, name="clowns_session_destroy")
            import :: c_int, c_ptr
            type(c_ptr), value :: s
        end function clowns_session_destroy
    end interface

contains

    ! The library's last error message as a Fortran string.
    function clowns_error_message() result(msg)
        character(len=:), allocatable :: msg
        character(kind=c_char), pointer :: cs(:)
        type(c_ptr) :: p
        integer :: n
        interface
            integer(c_size_t) function c_strlen(s) bind(C, name="strlen")
                import :: c_ptr, c_size_t
                type(c_ptr), value :: s
            end function c_strlen
        end interface
        p = clowns_last_error()
        n = int(c_strlen(p))
        call c_f_pointer(p, cs, [n])
        allocate(character(len=n) :: msg)
        msg = transfer(cs(1:n), msg)
    end function clowns_error_message

    ! Same call shape as the reference's PCGPME, for an explicit source-level swap
    ! inside cal_poisson_equation (1sub-momentum.F90:564).  Failures come back in
    ! ier as the reference's caller expects (non-zero, not 3000: icon = 911).
    subroutine pcgpme_via_gpu(alu, nl, mm2, llu, de, mnoe, n2, b, xe, eps1, parm, iter, ier)
        integer, intent(in) :: nl, mm2, mnoe, n2
        real*8, intent(inout) :: alu(mm2, nl), de(mnoe), b(mnoe), xe(mnoe + n2), eps1(2)
        integer, intent(inout) :: llu(mm2, nl), iter
        real*8, intent(in) :: parm
        integer, intent(out) :: ier
        call pcgpme_gpu(alu, nl, mm2, llu, de, mnoe, n2, b, xe, eps1, parm, iter, ier)
    end subroutine pcgpme_via_gpu

    ! Same call shape as the reference's PCGPME_WILL, for an explicit swap at
    ! 1sub-2DH-momentum.f90:325.  The reference has no error argument: with
    ! `status` present the library's return code comes back there (0 or a
    ! CLOWNS_ERR_* code; B is unchanged on failure); without it a failure stops
    ! the run with the library's message, as the reference stops on errors.
    subroutine pcgpme_will_via_gpu(al, nl, na, ll, d, n, n2, b, eps, parm, iter, status)
        integer, intent(in) :: nl, na, n, n2, iter
        real*8, intent(in) :: al(na, nl), d(n), eps, parm
        integer, intent(in) :: ll(na, nl)
        real*8, intent(inout) :: b(n)
        integer, intent(out), optional :: status
        integer(c_int) :: rc
        rc = pcgpme_will_gpu(al, nl, na, ll, d, n, n2, b, eps, parm, iter)
        if (present(status)) then
            status = rc
        else if (rc /= CLOWNS_OK) then
            write(6,*) 'PCGPME_WILL on the GPU failed: ', clowns_error_message()
            stop
        endif
    end subroutine pcgpme_will_via_gpu

end module clowns_gpu
