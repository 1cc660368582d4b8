"""The Fortran-subset translator (tests/golden/fortran_exec.py) that runs the
reference's routines for tests/golden/reference_runs.json, pinned on small
programs whose answers follow from the language's rules."""
import math
import pathlib
import sys

import pytest

sys.path.insert(0, str(pathlib.Path(__file__).resolve().parent / "golden"))

import fortran_exec as fx  # noqa: E402


def prog(src, defines=()):
    return fx.Program([src], set(defines))


def arr(kind, values, lb=1):
    return fx.FArray.from_list(kind, values, lb=(lb,))


def test_integer_arithmetic_truncates_toward_zero():
    p = prog("""
subroutine ints(a, b, q, r, s, t, u)
    implicit none
    integer, intent(in) :: a, b
    integer, intent(out) :: q, r, s, t
    real*8, intent(out) :: u
    q = a / b
    r = mod(a, b)
    s = sign(3, a)
    t = -7.9d0
    u = dfloat(a) ** 2
end subroutine
""")
    for a, b in ((7, 2), (-7, 2), (7, -2), (-7, -2)):
        _, _, q, r, s, t, u = p.call("ints", a, b, 0, 0, 0, 0, 0.0)
        assert q == int(a / b) and r == a - int(a / b) * b
        assert s == (3 if a >= 0 else -3) and t == -7 and u == float(a * a)


def test_do_variable_after_the_loop_and_trip_count():
    p = prog("""
subroutine loops(n, a, b, c, d, e)
    implicit none
    integer :: n, a, b, c, d, e, i, m
    do i = 1, n
    enddo
    a = i
    do i = 5, 1
    enddo
    b = i
    do i = 10, 1, -3
    enddo
    c = i
    do i = 1, 10
        if (i == 4) exit
    enddo
    d = i
    m = 3
    e = 0
    do i = 1, m
        m = 10
        e = e + 1
    enddo
end subroutine
""")
    r = p.call("loops", 4, 0, 0, 0, 0, 0)
    assert r[1:] == (5, 5, -2, 4, 3)


def test_sequence_association_and_aliasing():
    p = prog("""
subroutine fill(x, n, v)
    implicit none
    integer, intent(in) :: n
    real*8, intent(in) :: v
    real*8, dimension(n), intent(out) :: x
    integer :: i
    do i = 1, n
        x(i) = v + i
    enddo
end subroutine
subroutine shift(p, q, n)
    implicit none
    integer, intent(in) :: n
    real*8, dimension(n), intent(in) :: p
    real*8, dimension(n), intent(out) :: q
    integer :: i
    do i = 2, n
        q(i) = p(i - 1)
    enddo
end subroutine
subroutine top(wk, n)
    implicit none
    integer :: n
    real*8, dimension(n, 3) :: wk
    call fill(wk(1, 2), n, 10.0d0)
    call fill(wk, n, 0.0d0)
    call shift(wk(1, 2), wk(1, 2), n)
end subroutine
""")
    wk = fx.FArray.new("real", ((1, 4), (1, 3)), fill=-1.0)
    p.call("top", wk, 4)
    col = lambda j: [wk[i, j] for i in range(1, 5)]  # noqa: E731
    assert col(1) == [1.0, 2.0, 3.0, 4.0]
    # the aliased shift reads what it has just written: element 2 <- 1, 3 <- new 2, ...
    assert col(2) == [11.0, 11.0, 11.0, 11.0]
    assert col(3) == [-1.0] * 4


def test_scalar_copy_in_copy_out():
    p = prog("""
subroutine bump(a, b, c)
    implicit none
    integer, intent(inout) :: a
    integer, intent(in) :: b
    integer :: c
    a = a + 1
    c = c * 2
end subroutine
subroutine caller(x, v)
    implicit none
    integer :: x, k
    integer, dimension(3) :: v
    k = 5
    call bump(x, k, v(2))
    call bump(v(3), x + 1, x)
end subroutine
""")
    v = arr("int", [1, 2, 3])
    r = p.call("caller", 7, v)
    assert r[0] == 16 and v.to_list() == [1, 4, 4]


def test_initialised_locals_are_saved_and_hosts_are_shared():
    p = prog("""
subroutine counter(out)
    implicit none
    integer :: out
    integer :: n = 0
    n = n + 1
    call twice()
    out = n
contains
    subroutine twice()
        n = n * 2
    end subroutine
end subroutine
""")
    assert [p.call("counter", 0)[0] for _ in range(3)] == [2, 6, 14]


def test_goto_forward_backward_and_into_nested_blocks():
    p = prog("""
subroutine jumps(n, a, b, c)
    implicit none
    integer :: n, a, b, c, i, j
    a = 0
10  a = a + 1
    if (a < n) goto 10
    b = 0
    do i = 1, 6
        do j = 1, 3
            if (j == 2) goto 20
        enddo
        b = b + 100
20      continue
        if (i == 5) cycle
        b = b + 1
    enddo
    c = 0
    do i = 1, 10
        if (i > 3) goto 30
        c = c + i
    enddo
30  c = c * 10 + i
end subroutine
""")
    assert p.call("jumps", 4, 0, 0, 0)[1:] == (4, 5, 64)


def test_sections_constructors_and_reductions():
    p = prog("""
subroutine arrays(d, lg, m, loc, s, w)
    implicit none
    real*8, dimension(0:2, 4) :: d
    integer :: lg(0:2), loc, s, w, ix(0:2)
    real*8 :: m
    lg(0:2) = [ 7, 8, 9 ]
    m = minval(d(0:2:2, :), d(0:2:2, :) > 0.0d0)
    ix = 0
    ix(1) = -2
    ix(2) = 2
    loc = maxloc(abs(ix), 1)
    s = sum(abs(ix))
    w = sum(abs(ix(0:1)))
end subroutine
""")
    d = fx.FArray.new("real", ((0, 2), (1, 4)), fill=0.0)
    for (l, i), v in {(0, 1): 3.0, (1, 1): 0.5, (2, 2): 1.5, (0, 3): -1.0, (2, 4): 2.0}.items():
        d[l, i] = v
    lg = fx.FArray.new("int", ((0, 2),), fill=0)
    r = p.call("arrays", d, lg, 0.0, 0, 0, 0)
    assert lg.to_list() == [7, 8, 9]
    assert r[2:] == (1.5, 2, 4, 2)          # row 1 (0.5) is outside the section; maxloc: first maximum


def test_preprocessor_macros_sentinels_and_layout():
    src = """
#define SCALE_ 3
subroutine pp(a, b, c)
    implicit none
    integer :: a, b, c, nthr
#if defined(ALPHA) || defined(BETA)
    a = 1
#else
    a = 2
#endif
#ifndef GAMMA
    b = SCALE_ *      &
        & 2 ; c = 0
#endif
!$  nthr = omp_get_num_threads()
!$omp parallel do
    outer: do nthr = 1, 2
        c = c + nthr
    enddo outer
end subroutine
"""
    assert prog(src, {"BETA"}).call("pp", 0, 0, 0) == (1, 6, 3)
    assert prog(src).call("pp", 0, 0, 0) == (2, 6, 3)


def test_undefined_values_and_bounds_are_caught():
    p = prog("""
subroutine undef(x, r)
    implicit none
    real*8 :: x, r, t
    real*8, dimension(3) :: w
    r = w(2)
    x = t + 1.0d0
end subroutine
subroutine oob(v)
    implicit none
    integer, dimension(3) :: v
    v(4) = 1
end subroutine
""")
    with pytest.raises(TypeError):
        p.call("undef", 0.0, 0.0)
    with pytest.raises(IndexError):
        p.call("oob", arr("int", [0, 0, 0]))
    p2 = prog("""
subroutine undef2(r)
    implicit none
    real*8 :: r
    real*8, dimension(3) :: w
    r = w(2)
end subroutine
""")
    assert math.isnan(p2.call("undef2", 0.0)[0])


def test_unsupported_statements_leave_only_their_procedure_untranslated():
    p = prog("""
subroutine io()
    implicit none
    integer :: n
    read(5, *) n
end subroutine
subroutine fine(a)
    implicit none
    integer :: a
    a = a + 1
end subroutine
""")
    assert "io" in p.untranslated and p.call("fine", 1) == (2,)
    with pytest.raises(fx.FortranError):
        p.call("io")


def test_integer_powers_nint_and_labelled_end_do():
    p = prog("""
subroutine misc(n, a, b, c, d, s)
    implicit none
    integer :: n, c, d, s, k, j
    real*8 :: a, b
    a = 10d0**n
    b = 10d0**(-n)
    c = nint(2.5d0)
    d = nint(-2.5d0)
    s = 0
    do k = 1, 4
        do j = 1, 3
            if (j.eq.k) goto 400
            s = s + 1
400     end do
    end do
end subroutine
""")
    r = p.call("misc", 6, 0.0, 0.0, 0, 0, 0)
    assert r[1] == 1e6 and r[2] == 1.0 / 1e6          # a product, a reciprocal of a product
    assert r[3] == 3 and r[4] == -3                    # halves away from zero
    assert r[5] == 9                                   # 12 pairs less the 3 with j == k


def test_fixed_form_implicit_typing_and_characters():
    src = """C     a comment line
      subroutine last(text, nx, word, n2)
      character*12 text
      character*20 word
      do 100 n=12,1,-1
        if(text(n:n).ne.' ') then
          nx=n
          goto 200
        end if
  100 continue
  200 word = text(1:nx)//
     &  '.xyz'
      x = 2.5
      n2 = x * 3
      if (word(nx+1:nx+4) .eq. '.xyz  ') n2 = n2 + 100
      end
"""
    p = fx.Program([(src, True)], set())
    r = p.call("last", "abc/de", 0, "", 0)
    assert r[1] == 6 and r[2] == "abc/de.xyz".ljust(20) and r[3] == 107   # n2 = int(7.5) + 100


def test_unformatted_io_round_trip():
    p = prog("""
subroutine rw(n, m, x)
    implicit none
    integer :: n, m, i, j, ist
    real*8, dimension(0:2, 4) :: x
    open(9, file='t.bin', status='unknown', form='unformatted')
    write(9) n, (x(0, i), i = 1, 4)
    write(9) ((x(j, i), j = 0, 2), i = 1, 2)
    close(9)
    x = 0.0d0
    open(8, file='t.bin', status='old', form='unformatted')
    read(8) m, (x(1, i), i = 1, 4)
    read(8) x(0:2, 3), x(0, 4)
    read(8, iostat=ist) n
    m = m * 100 + ist
    close(8)
    open(8, file='none.bin', status='old', form='unformatted', err=50)
    m = -1
50  continue
end subroutine
""")
    p.env["_io"] = fx.FortranFiles()
    x = fx.FArray.new("real", ((0, 2), (1, 4)), fill=0.0)
    for l in range(3):
        for i in range(1, 5):
            x[l, i] = 10 * i + l
    r = p.call("rw", 7, 0, x)
    assert r[1] == 699                      # 7 read back, then the end of file: iostat -1
    assert [[x[l, i] for i in range(1, 5)] for l in range(3)] == [[0.0, 0.0, 10.0, 20.0], [10.0, 20.0, 11.0, 40.0],
                                                                  [0.0, 0.0, 12.0, 0.0]]
    recs = fx.FortranFiles.records(p.env["_io"].files["t.bin"])
    assert [len(r) for r in recs] == [4 + 32, 48] and recs[0][:4] == b"\x00\x00\x00\x07"   # big-endian
