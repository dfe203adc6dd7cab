!-----------------------------------------------------------------------------------------
! negf_gpu_shim.F90 - drop-in replacement of the reference's four hot-path subroutines.
!
! The reference calls, from Energy_Sweep (Source/Energy_Sweep.F90:28,40,42,45):
!     CALL Contact_Self_Energy ; CALL Get_Retarded_Greens ; CALL Calculate_Gnp ;
!     CALL Calculate_Observables
! with all data in NEGF_Module globals.  Linking this file instead of
! Contact_Self_Energy.o, Recursive_Greens.o, Calculate_Gnp.o and Calculate_Observables.o
! (Implement/Makefile:5) keeps Energy_Sweep.F90 unchanged: the subroutines below have the
! same names and no arguments, gather the module globals and call libnegf_gb300.so
! through ISO_C_BINDING (include/negf.h).  Link with  -L<dir> -lnegf_gb300.
!
! Behaviour kept from the reference: errorFlag receives the status code (INFO > 0 for a
! singular block, < 0 for library errors) and the run continues after printing it, as
! Source/Recursive_Greens.F90:28-33 does.  Energy_Sweep still assembles InvGRd on the
! host; the device rebuilds the same matrices from Htotd, energy and eta_sigma
! (Source/Energy_Sweep.F90:31-38), so InvGRd is not transferred.  Htotd/HopX are
! uploaded once per SCF iteration (when `ite` changes), which replaces MPI_Broadcast.
!
! No Fortran compiler exists in the build container; this file is provided as source.
!-----------------------------------------------------------------------------------------
MODULE negf_gpu_shim
    USE ISO_C_BINDING
    IMPLICIT NONE

    TYPE, BIND(C) :: negf_params_t
        INTEGER(C_INT32_T) :: npx, npy, npz, norb, n_hamiltonians, max_batch
        REAL(C_DOUBLE)     :: eta, sr_tol
        INTEGER(C_INT32_T) :: sr_max_iter, calc_spin, precision, device, mixed_slices, keep_g_columns
        INTEGER(C_INT32_T) :: residual_slices, sr_slices, calc_currents
        INTEGER(C_INT32_T) :: reserved(3)
        REAL(C_DOUBLE)     :: spin_ops(2, 4, 4, 3)   ! C order [3][4][4][2]
        INTEGER(C_INT32_T) :: contact_type, reserved1
        REAL(C_DOUBLE)     :: tunneling_rate, delta_sc(2), chi_lr
        REAL(C_DOUBLE)     :: gds(2, 4, 4)           ! C order [4][4][2]
        INTEGER(C_INT32_T) :: reserved2(8)
    END TYPE

    TYPE(C_PTR), SAVE :: negf_h = C_NULL_PTR
    INTEGER, SAVE     :: uploaded_ite = -1

    INTERFACE
        INTEGER(C_INT) FUNCTION negf_create(p, h) BIND(C, NAME="negf_create")
            IMPORT :: C_INT, C_PTR, negf_params_t
            TYPE(negf_params_t), INTENT(IN) :: p
            TYPE(C_PTR), INTENT(OUT)        :: h
        END FUNCTION
        INTEGER(C_INT) FUNCTION negf_set_hamiltonian(h, slot, htotd, hopx) BIND(C, NAME="negf_set_hamiltonian")
            IMPORT :: C_INT, C_INT32_T, C_PTR, C_DOUBLE_COMPLEX
            TYPE(C_PTR), VALUE                  :: h
            INTEGER(C_INT32_T), VALUE           :: slot
            COMPLEX(C_DOUBLE_COMPLEX), INTENT(IN) :: htotd(*), hopx(*)
        END FUNCTION
        INTEGER(C_INT) FUNCTION negf_contact_self_energy(h, e, sl, sr, gl, gr, dosc) &
                BIND(C, NAME="negf_contact_self_energy")
            IMPORT :: C_INT, C_PTR, C_DOUBLE, C_DOUBLE_COMPLEX
            TYPE(C_PTR), VALUE      :: h
            REAL(C_DOUBLE), VALUE   :: e
            COMPLEX(C_DOUBLE_COMPLEX) :: sl(*), sr(*), gl(*), gr(*)
            REAL(C_DOUBLE)          :: dosc(2)
        END FUNCTION
        INTEGER(C_INT) FUNCTION negf_get_retarded_greens(h) BIND(C, NAME="negf_get_retarded_greens")
            IMPORT :: C_INT, C_PTR
            TYPE(C_PTR), VALUE :: h
        END FUNCTION
        INTEGER(C_INT) FUNCTION negf_calculate_gnp(h, f1, f2, de, rhon, rhop) BIND(C, NAME="negf_calculate_gnp")
            IMPORT :: C_INT, C_PTR, C_DOUBLE
            TYPE(C_PTR), VALUE    :: h
            REAL(C_DOUBLE), VALUE :: f1, f2, de
            REAL(C_DOUBLE)        :: rhon(*), rhop(*)
        END FUNCTION
        ! an absent OPTIONAL dummy of a BIND(C) interface is passed as a null pointer
        ! (Fortran 2018, 18.3.6), which is what the C entry points take for "not wanted"
        INTEGER(C_INT) FUNCTION negf_calculate_observables(h, de, f1, f2, t12, eden, hden, modes, cc, sx, sy, sz) &
                BIND(C, NAME="negf_calculate_observables")
            IMPORT :: C_INT, C_PTR, C_DOUBLE
            TYPE(C_PTR), VALUE    :: h
            REAL(C_DOUBLE), VALUE :: de, f1, f2
            REAL(C_DOUBLE)        :: t12, eden, hden, modes(2), cc(2)
            REAL(C_DOUBLE), OPTIONAL :: sx(*), sy(*), sz(*)
        END FUNCTION
        INTEGER(C_INT) FUNCTION negf_calculate_currents(h, jx, jy, jz) BIND(C, NAME="negf_calculate_currents")
            IMPORT :: C_INT, C_PTR, C_DOUBLE
            TYPE(C_PTR), VALUE    :: h
            REAL(C_DOUBLE)        :: jx(*), jy(*), jz(*)
        END FUNCTION
        INTEGER(C_INT) FUNCTION negf_calculate_resolved(h, erjx, erjy, erjz, errhon, orjx, orjy, orjz, orrhon) &
                BIND(C, NAME="negf_calculate_resolved")
            IMPORT :: C_INT, C_PTR, C_DOUBLE
            TYPE(C_PTR), VALUE    :: h
            REAL(C_DOUBLE), OPTIONAL :: erjx(*), erjy(*), erjz(*), errhon(*), orjx(*), orjy(*), orjz(*), orrhon(*)
        END FUNCTION
    END INTERFACE

CONTAINS

    SUBROUTINE negf_shim_check(code, what)
        USE NEGF_Module, ONLY: errorFlag, energy
        INTEGER(C_INT), INTENT(IN) :: code
        CHARACTER(*), INTENT(IN)   :: what
        IF (code /= 0) THEN
            WRITE(*,*) "ERROR in ", what, ": status = ", code, " Energy = ", energy
            errorFlag = code
        ENDIF
    END SUBROUTINE

    SUBROUTINE negf_shim_init
        USE NEGF_Module
        TYPE(negf_params_t) :: p
        INTEGER(C_INT)      :: st
        IF (C_ASSOCIATED(negf_h) .AND. uploaded_ite == ite) RETURN
        IF (.NOT. C_ASSOCIATED(negf_h)) THEN
            p%npx = Npx; p%npy = Npy; p%npz = Npz; p%norb = Norb
            p%n_hamiltonians = 1; p%max_batch = 1
            p%eta = eta_sigma; p%sr_tol = 1D-8; p%sr_max_iter = 20000
            p%calc_spin = calcSigExp; p%precision = 0; p%device = 0
            p%mixed_slices = 0; p%keep_g_columns = 0; p%reserved = 0
            p%residual_slices = 0; p%sr_slices = 0; p%calc_currents = 1
            p%spin_ops = 0D0
            ! contacts (Source/Read_In_Allocate.F90:19,69-76); gds = 0 selects the model's gDS
            p%contact_type = contactType; p%reserved1 = 0; p%reserved2 = 0
            p%tunneling_rate = 1D0; p%delta_sc = 0D0; p%chi_lr = 0D0; p%gds = 0D0
            IF (contactType == 3) THEN
                p%delta_sc(1) = DeltaSCL; p%delta_sc(2) = DeltaSCR; p%chi_lr = chiLR
            ENDIF
            st = negf_create(p, negf_h)
            IF (st /= 0) STOP "negf_create failed"
        ENDIF
        st = negf_set_hamiltonian(negf_h, 0_C_INT32_T, Htotd, HopX)
        CALL negf_shim_check(st, "negf_set_hamiltonian")
        uploaded_ite = ite
    END SUBROUTINE

END MODULE negf_gpu_shim


SUBROUTINE Contact_Self_Energy
    USE NEGF_Module
    USE negf_gpu_shim
    IMPLICIT NONE
    REAL(C_DOUBLE) :: dosc(2)
    INTEGER(C_INT) :: st
    CALL negf_shim_init
    st = negf_contact_self_energy(negf_h, energy, SigmaL, SigmaR, GammaL, GammaR, dosc)
    CALL negf_shim_check(st, "Contact_Self_Energy")
    DOSc1(eCtr+1) = DOSc1(eCtr+1) + dosc(1)
    DOSc2(eCtr+1) = DOSc2(eCtr+1) + dosc(2)
END SUBROUTINE Contact_Self_Energy


SUBROUTINE Get_Retarded_Greens
    USE NEGF_Module
    USE negf_gpu_shim
    IMPLICIT NONE
    INTEGER(C_INT) :: st
    st = negf_get_retarded_greens(negf_h)
    CALL negf_shim_check(st, "Get_Retarded_Greens")
END SUBROUTINE Get_Retarded_Greens


SUBROUTINE Calculate_Gnp
    USE NEGF_Module
    USE negf_gpu_shim
    IMPLICIT NONE
    INTEGER(C_INT) :: st
    st = negf_calculate_gnp(negf_h, f1, f2, deltaE, RhoN, RhoP)
    CALL negf_shim_check(st, "Calculate_Gnp")
    ! energy- and orbital-resolved densities (Source/Calculate_Gnp.F90:125-129)
    IF (erCD == 1) THEN
        st = negf_calculate_resolved(negf_h, errhon=ERRhon(:, :, :, eCtr+1))
        CALL negf_shim_check(st, "Calculate_Gnp (ERRhon)")
    ENDIF
    IF (orCD == 1) THEN
        st = negf_calculate_resolved(negf_h, orrhon=ORRhon)
        CALL negf_shim_check(st, "Calculate_Gnp (ORRhon)")
    ENDIF
END SUBROUTINE Calculate_Gnp


SUBROUTINE Calculate_Observables
    USE NEGF_Module
    USE negf_gpu_shim
    IMPLICIT NONE
    INTEGER(C_INT) :: st
    REAL(C_DOUBLE) :: t, ed, hd, modes(2)
    IF (calcSigExp == 1) THEN
        st = negf_calculate_observables(negf_h, deltaE, f1, f2, t, ed, hd, modes, ContactCurrent, &
                                        SigXExp, SigYExp, SigZExp)
    ELSE
        st = negf_calculate_observables(negf_h, deltaE, f1, f2, t, ed, hd, modes, ContactCurrent)
    ENDIF
    CALL negf_shim_check(st, "Calculate_Observables")
    T12(eCtr+1) = T12(eCtr+1) + t
    EDensity(eCtr+1) = EDensity(eCtr+1) + ed
    HDensity(eCtr+1) = HDensity(eCtr+1) + hd
    Modec1(eCtr+1) = Modec1(eCtr+1) + modes(1)
    Modec2(eCtr+1) = Modec2(eCtr+1) + modes(2)
    ! bond currents (Source/Calculate_Observables.F90:110-169)
    st = negf_calculate_currents(negf_h, Jx, Jy, Jz)
    CALL negf_shim_check(st, "Calculate_Observables (currents)")
    ! energy- and orbital-resolved current densities (:124-160); ERJx(:,:,:,eCtr+1) is
    ! contiguous, so the library adds into the caller's column in place
    IF (erCD == 1) THEN
        st = negf_calculate_resolved(negf_h, erjx=ERJx(:, :, :, eCtr+1), erjy=ERJy(:, :, :, eCtr+1), &
                                     erjz=ERJz(:, :, :, eCtr+1))
        CALL negf_shim_check(st, "Calculate_Observables (ERCD)")
    ENDIF
    IF (orCD == 1) THEN
        st = negf_calculate_resolved(negf_h, orjx=ORJx, orjy=ORJy, orjz=ORJz)
        CALL negf_shim_check(st, "Calculate_Observables (ORCD)")
    ENDIF
END SUBROUTINE Calculate_Observables
