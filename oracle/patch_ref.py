#!/usr/bin/env python3
"""Mechanical build fixes that let the 2002-era BlochLib reference compile with g++ 13.

Test infrastructure only: this script prepares a scratch copy of the reference's
sources (never committed) so that the reference itself can be executed as the oracle
that pins this repository's CPU restatement and golden FID fixtures.

Usage: patch_ref.py <scratch_src_dir>

Every edit is an exact-text replacement whose expected match count is asserted, so a
changed reference tree fails loudly instead of being patched silently.  None of the
edits changes the arithmetic of the powder-FID path except the last one, which turns
the precision of the QL eigen-iteration into a macro (BL_QL_REAL, default float as
shipped) so that a second, all-double build can be made with -DBL_QL_REAL=double.
"""
import re
import sys
from pathlib import Path


def sub(root, rel, old, new, count=1, regex=False):
    p = root / rel
    txt = p.read_text(encoding="latin-1")
    if regex:
        out, n = re.subn(old, new, txt, flags=re.S)
    else:
        n = txt.count(old)
        out = txt.replace(old, new)
    if count is not None and n != count:
        raise SystemExit(f"patch_ref: {rel}: expected {count} match(es) of {old!r}, found {n}")
    if n == 0 and count is None:
        raise SystemExit(f"patch_ref: {rel}: no match of {old!r}")
    p.write_text(out, encoding="latin-1")


def main():
    root = Path(sys.argv[1])
    # matfft.h: the fft()/ifft() wrappers call FFT/IFFT templates declared later in the
    # file; two-phase lookup needs them declared first.
    sub(root, "container/matrix/matfft.h",
        "//various 'auxilliarly names' for the FFT\n",
        "template<class nt1, class st1> _matrix<complex, FullMatrix> FFT(const _matrix<nt1, st1> &in);\n"
        "template<class nt1, class st1> _matrix<complex, FullMatrix> IFFT(const _matrix<nt1, st1> &in);\n"
        "//various 'auxilliarly names' for the FFT\n")
    # functions the headers place in BlochLib but call through std::
    for rel in ["container/matrix/LU.h", "container/matrix/matdiagonalize.h", "container/matrix/matqr.h"]:
        sub(root, rel, r"std::(solve|PackedQR|UnPackQR|eigenvalues|diag)\(", r"::BlochLib::\1(",
            count=None, regex=True)
    # matqr.h: never-instantiated overloads refer to an undeclared 'coief'
    sub(root, "container/matrix/matqr.h", "\tcoief.resize(a.rows());\n\tcoief.fill(a.rows());\n",
        "\n", count=2)
    # matexp.h: a never-instantiated overload uses an undeclared 'mul'
    sub(root, "container/matrix/matexp.h", "\tdia=exp(mul*dia);\n\treturn prop(U,dia);\n\t//return PadeSeries(in);",
        "\tdia=exp(dia);\n\treturn prop(U,dia);\n\t//return PadeSeries(in);")
    # matdiagonalize.h: 'sign' used before its definition
    txt = (root / "container/matrix/matdiagonalize.h").read_text(encoding="latin-1")
    first_tpl = txt.index("BEGIN_BL_NAMESPACE")
    fwd = ("BEGIN_BL_NAMESPACE\ntemplate<class nt1, class nt2> inline OutType(nt1, nt2) sign(nt1 a, nt2 b);\n")
    txt = txt[:first_tpl] + fwd + txt[first_tpl + len("BEGIN_BL_NAMESPACE\n"):]
    (root / "container/matrix/matdiagonalize.h").write_text(txt, encoding="latin-1")
    # complex.h: norm() used by operator< before it is declared
    sub(root, "container/complex.h",
        "template<class Ctype_T>\ninline bool Complex<Ctype_T>::operator<(",
        "template<class C> inline C norm(const Complex<C>&);\n"
        "template<class Ctype_T>\ninline bool Complex<Ctype_T>::operator<(")
    # no cblas/ATLAS in this toolchain: use the bundled PHiPAC GEMM kernels
    sub(root, "blochconfig.h", "#define AUX_BLAS_LIB 1", "/* #undef AUX_BLAS_LIB */")
    # non-BLAS adjprop fallback names the wrong argument
    sub(root, "container/matrix/matmat.h", "\t(*this)=adjoint(A)*(*this)*(m1);\n", "\t(*this)=adjoint(A)*(*this)*(A);\n")
    sub(root, "container/matrix/matdiagonalize.h", "\tBL_NAMESPACE::diag((*this), dia, U, des);",
        "\t::BlochLib::diag((*this), dia, U, des);", count=2)
    # dgemm.h: DGEMM wrappers call the dgemm_ template defined further down
    sub(root, "container/matrix/dgemm.h",
        "template<class T,class T1, class T2>\nvoid DGEMM(char *transA, char *transB,",
        "template<class T,class T1, class T2>\nvoid dgemm_(char *transA, char *transB, int *M, int *N, int *K,"
        " T1 *alpha, T* A, int *Astride, T* B, int *Bstride, T2 *beta, T* C, int *Cstride);\n"
        "template<class T,class T1, class T2>\nvoid DGEMM(char *transA, char *transB,", count=None)
    # grids/coords.h (pulled in by utils and mpi headers)
    sub(root, "container/grids/coords.h", "inline coord<T1,N1> alterSize(int N1)", "inline coord<T1,N1> alterSize()")
    sub(root, "container/grids/coords.h",
        r"void Rotate2D\(double theta\)\{.*?tz\*\(cps\*sth\);\n\t\t\}",
        "void Rotate2D(double theta){ }", count=1, regex=True)
    sub(root, "container/grids/coords.h",
        "inline coord<T,N> &coord<T,N>::operator=(const coord<T1,N> &rhs)\n{\n\t//TheType=rhs.TheType;\n"
        "    (*this) = VExpr<typename coord<T1, N>::const_iterator>(x.const_iter());",
        "inline coord<T,N> &coord<T,N>::operator=(const coord<T1,N> &rhs)\n{\n\t//TheType=rhs.TheType;\n"
        "    (*this) = VExpr<typename coord<T1, N>::const_iterator>(rhs.const_iter());")
    sub(root, "container/grids/coords.h",
        "inline coord<T,N>& coord<T,N>::operator OP (const Vector<T1> &in)\t\\\n\t\t{\t\\\n"
        "\t\t\t(*this) OP VExpr<typename coord<T1, N>::const_iterator>(x.const_iter());",
        "inline coord<T,N>& coord<T,N>::operator OP (const Vector<T1> &in)\t\\\n\t\t{\t\\\n"
        "\t\t\t(*this) OP VExpr<typename coord<T1, N>::const_iterator>(in.const_iter());")
    # comparisons NUM-op-coord index the scalar instead of the coord
    p = root / "container/grids/coords.h"
    txt = p.read_text(encoding="latin-1")
    txt, n = re.subn(r"(const NUM & a, const coord<T1,N> & b\)[^}]*?if\()a\[i\] (\S+) b\)",
                     r"\1a \2 b[i])", txt, flags=re.S)
    if n != 6:
        raise SystemExit(f"patch_ref: coords.h NUM-op-coord: expected 6, found {n}")
    p.write_text(txt, encoding="latin-1")
    sub(root, "container/grids/grids.h", "oo<<myIt.Point()<<endl;", "oo<<myIt.Point()<<std::endl;", count=None)
    sub(root, "container/grids/unigrid.h", "class UniforGridIter;", "class UniformGridIter;")
    sub(root, "container/grids/xyzshape.h", "NonShape::operator=(in);", "NonShape::operator=(rhs);", count=3)
    # utils
    sub(root, "utils/random.h", r"std::(PoissonRand|GaussianRand)\(", r"BL_NAMESPACE::\1(", count=None, regex=True)
    sub(root, "utils/matlab5.h", "case miUINT8:", "case 2:", count=2)
    sub(root, "utils/matlab5.h", "case miDOUBLE:", "case 9:", count=2)
    # precision of the QL iteration of the Hermitian eigensolver becomes a macro
    sub(root, "container/matrix/matdiagonalize.h",
        "\tfloat dd;\n\tfloat s,r,p,g,f,c,b;\n\tfloat x;\n",
        "\tBL_QL_REAL dd;\n\tBL_QL_REAL s,r,p,g,f,c,b;\n\tBL_QL_REAL x;\n")
    sub(root, "container/matrix/matdiagonalize.h", "\tVector<float> e(n);\n", "\tVector<BL_QL_REAL> e(n);\n")


if __name__ == "__main__":
    main()
