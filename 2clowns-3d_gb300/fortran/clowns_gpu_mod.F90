!%%%%%%%%%%%%%%%%%%%%% FILE: clowns_gpu_mod.F90 %%%%%%%%%%%%%%%%%%%%%%%%%%%%%%%%
! ISO_C_BINDING interface to libclowns_gpu.so (the GB300 pressure solve).
!
! Two ways to use it from the model:
!
!  1. Link-level drop-in: link libclowns_gpu.so instead of pcgpme_para.o.  The
!     library exports the symbol pcgpme_ (ifort's name for PCGPME), so
!     cal_poisson_equation keeps calling PCGPME(alu,nl,mm2,llu,de,mnoe,64,b,
!     xe(1:mm2),eps1,parm,iter,ier) unchanged.
!
!  2. Explicit calls through the interfaces below, e.g. the device-resident
!     entry points when the module arrays are kept on the GPU by the host code.
!
! The assembly, classification, right-hand side and correction entry points
! take the module arrays of `arrays` explicitly (Fortran module descriptors are
! compiler-specific, so only raw arrays cross the boundary).  The derived type
! cellflag is passed as two integer arrays nff(:)%f and nff(:)%b.
!
! This file is not compiled in this repository (no Fortran compiler is
! available where it was written); it documents the binding a maintainer adds.
module clowns_gpu
    use iso_c_binding
    implicit none

    type, bind(C) :: clowns_solve_info
        real(c_double) :: eps, bn
        integer(c_int) :: iter, ier, reason, outer
    end type clowns_solve_info

    interface
        ! PCGPME drop-in with host arrays (same arguments, by reference)
        subroutine pcgpme_gpu(al, nl, na, ll, d, n, n2, b, x, eps, parm, iter, ier) &
                bind(C, name="pcgpme_gpu")
            import :: c_double, c_int
            real(c_double), intent(inout) :: al(*), d(*), b(*), x(*), eps(2)
            integer(c_int), intent(in) :: nl, na, n, n2
            integer(c_int), intent(inout) :: ll(*), iter
            real(c_double), intent(in) :: parm
            integer(c_int), intent(out) :: ier
        end subroutine pcgpme_gpu

        ! PCGPME_WILL drop-in (2DH dispersion solve) with host arrays; B in: RHS,
        ! out: what the reference leaves in B.  Returns 0 or a CLOWNS_ERR_* code.
        integer(c_int) function pcgpme_will_gpu(al, nl, na, ll, d, n, n2, b, eps, parm, iter) &
                bind(C, name="pcgpme_will_gpu")
            import :: c_double, c_int
            real(c_double), intent(in) :: al(*), d(*), eps, parm
            integer(c_int), intent(in) :: nl, na, n, n2, iter, ll(*)
            real(c_double), intent(inout) :: b(*)
        end function pcgpme_will_gpu

        ! Device-resident solve: device addresses and a device workspace
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
            type(clowns_solve_info) :: info
        end function clowns_pcgpme_dev

        ! Allocation-free device solve (n <= 32768)
        integer(c_int) function clowns_pcgpme_static_dev(al, nl, na, ll, d, n, b, x, eps, parm, &
                iter, stream, info) bind(C, name="clowns_pcgpme_static_dev")
            import :: c_int, c_double, c_ptr, clowns_solve_info
            type(c_ptr), value :: al, ll, d, b, x, stream
            integer(c_int), value :: nl, na, n, iter
            real(c_double), value :: eps, parm
            type(clowns_solve_info) :: info
        end function clowns_pcgpme_static_dev

        ! cal_matrix_element on device arrays
        integer(c_int) function clowns_assemble_dev(dims, inne, inne2, mx2, in, jn, kn, nf, nfb, &
                x, dx, sp, ifln, fln, mno, alu_c, ll_c, de_c, mm2, alu, llu, de, err_cell, stream) &
                bind(C, name="clowns_assemble_dev")
            import :: c_int, c_ptr
            integer(c_int), intent(in) :: dims(6)
            integer(c_int), value :: inne, inne2, mx2, ifln, mm2
            type(c_ptr), value :: in, jn, kn, nf, nfb, x, dx, sp, fln, mno, alu_c, ll_c, de_c
            type(c_ptr), value :: alu, llu, de, err_cell, stream
        end function clowns_assemble_dev

        ! const char*: convert with c_f_pointer for printing
        type(c_ptr) function clowns_last_error() bind(C, name="clowns_last_error")
            import :: c_ptr
        end function clowns_last_error
    end interface

contains

    ! Same call shape as the reference's PCGPME, for an explicit source-level swap
    ! inside cal_poisson_equation (1sub-momentum.F90:564).
    subroutine pcgpme_via_gpu(alu, nl, mm2, llu, de, mnoe, n2, b, xe, eps1, parm, iter, ier)
        integer, intent(in) :: nl, mm2, mnoe, n2
        real*8, intent(inout) :: alu(mm2, nl), de(mnoe), b(mnoe), xe(mnoe + n2), eps1(2)
        integer, intent(inout) :: llu(mm2, nl), iter
        real*8, intent(in) :: parm
        integer, intent(out) :: ier
        call pcgpme_gpu(alu, nl, mm2, llu, de, mnoe, n2, b, xe, eps1, parm, iter, ier)
    end subroutine pcgpme_via_gpu

    ! Same call shape as the reference's PCGPME_WILL, for an explicit swap at
    ! 1sub-2DH-momentum.f90:325.
    subroutine pcgpme_will_via_gpu(al, nl, na, ll, d, n, n2, b, eps, parm, iter)
        integer, intent(in) :: nl, na, n, n2, iter
        real*8, intent(in) :: al(na, nl), d(n), eps, parm
        integer, intent(in) :: ll(na, nl)
        real*8, intent(inout) :: b(n)
        integer(c_int) :: rc
        rc = pcgpme_will_gpu(al, nl, na, ll, d, n, n2, b, eps, parm, iter)
    end subroutine pcgpme_will_via_gpu

end module clowns_gpu
