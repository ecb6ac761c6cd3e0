// P/Invoke declarations of libddla_gb300 (include/ddla_gb300.h) for DDLA.
//
// The sibling of DDLA's BLIS binding (DDLA/BLAS/Native/3m.cs:12-162,
// `public static partial class Source` with [DllImport(BlisDLL, ...)]): the
// BLIS-shaped calls keep BLIS's argument lists (dim_t / inc_t are long, flags
// are DDLA's int enums, alpha / beta by `in double`, matrices as
// `ref double` head element plus row and column strides) and return an int
// status instead of void.  The factorization-level calls keep DDLA's
// conventions (relative LU pivots, LU.cs:367-374).  Host pointers only: every
// call copies to the GPU, computes and copies back before it returns, so the
// marshaller's pinning for the duration of the call is all that is needed.
//
// tests/test_csharp_binding.py checks every [DllImport] below against the C
// prototypes of include/ddla_gb300.h (name, parameter count, parameter kinds).
using System;
using System.Runtime.InteropServices;
using DDLA.Core;
using DDLA.Misc.Flags;

namespace DDLA.BLAS.Cuda;

public static partial class Source
{
    public const string Lib = "ddla_gb300";

    // ------------------------------------------------------------ runtime

    [DllImport(Lib, EntryPoint = "ddla_last_error")]
    static extern IntPtr LastErrorPtr();
    [DllImport(Lib, EntryPoint = "ddla_version")]
    static extern IntPtr VersionPtr();
    [DllImport(Lib, EntryPoint = "ddla_kernel_launches")]
    public static extern long KernelLaunches();
    // tuning keys ("lu.nb", "panel.cluster", ...; no DDLA counterpart)
    [DllImport(Lib, EntryPoint = "ddla_tune_set")]
    public static extern int TuneSet(string key, long value);
    [DllImport(Lib, EntryPoint = "ddla_tune_get")]
    public static extern long TuneGet(string key, long dflt);

    public static string LastError() => Marshal.PtrToStringAnsi(LastErrorPtr()) ?? "";
    public static string Version() => Marshal.PtrToStringAnsi(VersionPtr()) ?? "";

    // ------------------------------------------------------------ level 3 (BLIS-shaped)

    // replaces bli_dgemm, DDLA/BLAS/Native/3m.cs:12-24
    [DllImport(Lib, EntryPoint = "ddla_dgemm")]
    public static extern int GeMM(TransType transa, TransType transb, dim_t m, dim_t n, dim_t k,
        in double alpha, ref double a, inc_t rsa, inc_t csa, ref double b, inc_t rsb, inc_t csb,
        in double beta, ref double c, inc_t rsc, inc_t csc);

    // replaces bli_dgemmt, 3m.cs:26-38
    [DllImport(Lib, EntryPoint = "ddla_dgemmt")]
    public static extern int GeMMT(UpLo uploc, TransType transa, TransType transb, dim_t m, dim_t k,
        in double alpha, ref double a, inc_t rsa, inc_t csa, ref double b, inc_t rsb, inc_t csb,
        in double beta, ref double c, inc_t rsc, inc_t csc);

    // replaces bli_dsyrk, 3m.cs:96-106
    [DllImport(Lib, EntryPoint = "ddla_dsyrk")]
    public static extern int SyRk(UpLo uploc, TransType transa, dim_t m, dim_t k,
        in double alpha, ref double a, inc_t rsa, inc_t csa, in double beta, ref double c, inc_t rsc, inc_t csc);

    // replaces bli_dsymm, 3m.cs:81-94
    [DllImport(Lib, EntryPoint = "ddla_dsymm")]
    public static extern int SyMM(SideType sidea, UpLo uploa, ConjType conja, TransType transb, dim_t m, dim_t n,
        in double alpha, ref double a, inc_t rsa, inc_t csa, ref double b, inc_t rsb, inc_t csb,
        in double beta, ref double c, inc_t rsc, inc_t csc);

    // replaces bli_dsyr2k, 3m.cs:108-120
    [DllImport(Lib, EntryPoint = "ddla_dsyr2k")]
    public static extern int SyR2k(UpLo uploc, TransType transa, TransType transb, dim_t m, dim_t k,
        in double alpha, ref double a, inc_t rsa, inc_t csa, ref double b, inc_t rsb, inc_t csb,
        in double beta, ref double c, inc_t rsc, inc_t csc);

    // replaces bli_dtrmm, 3m.cs:122-133
    [DllImport(Lib, EntryPoint = "ddla_dtrmm")]
    public static extern int TrMM(SideType sidea, UpLo uploa, TransType transa, DiagType diaga, dim_t m, dim_t n,
        in double alpha, ref double a, inc_t rsa, inc_t csa, ref double b, inc_t rsb, inc_t csb);

    // replaces bli_dtrmm3, 3m.cs:135-149
    [DllImport(Lib, EntryPoint = "ddla_dtrmm3")]
    public static extern int TrMM3(SideType sidea, UpLo uploa, TransType transa, DiagType diaga, TransType transb,
        dim_t m, dim_t n, in double alpha, ref double a, inc_t rsa, inc_t csa, ref double b, inc_t rsb, inc_t csb,
        in double beta, ref double c, inc_t rsc, inc_t csc);

    // replaces bli_dtrsm, 3m.cs:151-162
    [DllImport(Lib, EntryPoint = "ddla_dtrsm")]
    public static extern int TrSM(SideType side, UpLo uploa, TransType transa, DiagType diaga, dim_t m, dim_t n,
        in double alpha, ref double a, inc_t rsa, inc_t csa, ref double b, inc_t rsb, inc_t csb);

    // ------------------------------------------------------------ factorizations

    /// <summary>ddla_opts: zero means the library's defaults.</summary>
    [StructLayout(LayoutKind.Sequential)]
    public struct Opts
    {
        public int Precision, Nb, MaxIter, Reserved;
        public double Tol;
    }

    /// <summary>ddla_solve_report of the mixed-precision solves.</summary>
    [StructLayout(LayoutKind.Sequential)]
    public struct SolveReport
    {
        public int Iterations, Converged, Precision, Info;
        public double BackwardError, ForwardError, FactorMs, RefineMs;
        public int PivotsAgree, PivotsFirstDiff;
        public double Growth, DiagRatio;
    }

    public const int PrecFP64 = 0, PrecFP32 = 1, PrecTF32x3 = 2, PrecBF16x3 = 3, PrecOzaki = 4;

    // LU.PLUDecompose / PLUSolve (DDLA/Factorizations/LU.cs:251-287): relative pivots, as DDLA
    [DllImport(Lib, EntryPoint = "ddla_dgetrf")]
    public static extern int GetRF(dim_t n, ref double a, inc_t rsa, inc_t csa, ref int piv, in Opts opts);
    [DllImport(Lib, EntryPoint = "ddla_dgetrs")]
    public static extern int GetRS(int trans, dim_t n, dim_t nrhs, ref double lu, inc_t rsa, inc_t csa,
        ref int piv, ref double b, inc_t rsb, inc_t csb);
    // LU.LUDecompose / LUSolve (LU.cs:130-232)
    [DllImport(Lib, EntryPoint = "ddla_dgetrf_nopiv")]
    public static extern int GetRFNoPiv(dim_t n, ref double a, inc_t rsa, inc_t csa, in Opts opts);
    [DllImport(Lib, EntryPoint = "ddla_dgetrs_nopiv")]
    public static extern int GetRSNoPiv(int trans, dim_t n, dim_t nrhs, ref double lu, inc_t rsa, inc_t csa,
        ref double b, inc_t rsb, inc_t csb);
    // Cholesky.CholDecompose / CholeskySolve (Cholesky.cs:52-123)
    [DllImport(Lib, EntryPoint = "ddla_dpotrf")]
    public static extern int PotRF(UpLo uplo, dim_t n, ref double a, inc_t rsa, inc_t csa, in Opts opts);
    [DllImport(Lib, EntryPoint = "ddla_dpotrs")]
    public static extern int PotRS(UpLo uplo, dim_t n, dim_t nrhs, ref double a, inc_t rsa, inc_t csa,
        ref double b, inc_t rsb, inc_t csb);
    // LDLT.LDLTDecompose / LDLTSolve (LDLT.cs:56-126)
    [DllImport(Lib, EntryPoint = "ddla_dldlt")]
    public static extern int LDLT(UpLo uplo, dim_t n, ref double a, inc_t rsa, inc_t csa, in Opts opts);
    [DllImport(Lib, EntryPoint = "ddla_dldlts")]
    public static extern int LDLTS(UpLo uplo, dim_t n, dim_t nrhs, ref double a, inc_t rsa, inc_t csa,
        ref double b, inc_t rsb, inc_t csb);

    // mixed precision + FP64 refinement (no DDLA counterpart: DDLA's solves are FP64 only);
    // xRef may be IntPtr.Zero (no forward error)
    [DllImport(Lib, EntryPoint = "ddla_dgesv_mixed")]
    public static extern int GeSVMixed(dim_t n, dim_t nrhs, ref double a, inc_t rsa, inc_t csa,
        ref double b, inc_t rsb, inc_t csb, ref double x, inc_t rsx, inc_t csx,
        IntPtr xRef, in Opts opts, out SolveReport report);
    [DllImport(Lib, EntryPoint = "ddla_dposv_mixed")]
    public static extern int PoSVMixed(UpLo uplo, dim_t n, dim_t nrhs, ref double a, inc_t rsa, inc_t csa,
        ref double b, inc_t rsb, inc_t csb, ref double x, inc_t rsx, inc_t csx,
        IntPtr xRef, in Opts opts, out SolveReport report);
    [DllImport(Lib, EntryPoint = "ddla_dsysv_mixed")]
    public static extern int SySVMixed(UpLo uplo, dim_t n, dim_t nrhs, ref double a, inc_t rsa, inc_t csa,
        ref double b, inc_t rsb, inc_t csb, ref double x, inc_t rsx, inc_t csx,
        IntPtr xRef, in Opts opts, out SolveReport report);

    // ------------------------------------------------------------ QR and reductions

    // QR.QRDecompose(A, T) (DDLA/Factorizations/QR.cs:130-149): same storage of R, the
    // Householder vectors and T, so DDLA's ApplyQ / FormQ / Solve also work on the result
    [DllImport(Lib, EntryPoint = "ddla_dgeqrf")]
    public static extern int GeQRF(dim_t m, dim_t n, ref double a, inc_t rsa, inc_t csa,
        ref double t, dim_t tRows, inc_t rst, inc_t cst, in Opts opts);
    // QR.ApplyQ / ApplyQT (QR.cs:79-109); trans != 0 applies Q^T
    [DllImport(Lib, EntryPoint = "ddla_dormqr")]
    public static extern int OrMQR(int trans, dim_t m, dim_t n, dim_t nrhs, ref double a, inc_t rsa, inc_t csa,
        ref double t, dim_t tRows, inc_t rst, inc_t cst, ref double b, inc_t rsb, inc_t csb);
    // QR.Solve (QR.cs:151-168), least squares for m >= n
    [DllImport(Lib, EntryPoint = "ddla_dgeqrs")]
    public static extern int GeQRS(dim_t m, dim_t n, dim_t nrhs, ref double a, inc_t rsa, inc_t csa,
        ref double t, dim_t tRows, inc_t rst, inc_t cst, ref double b, inc_t rsb, inc_t csb,
        ref double x, inc_t rsx, inc_t csx);
    // QR.FormQ(A, T, Q) (QR.cs:179-201)
    [DllImport(Lib, EntryPoint = "ddla_dorgqr")]
    public static extern int OrGQR(dim_t m, dim_t n, ref double a, inc_t rsa, inc_t csa,
        ref double t, dim_t tRows, inc_t rst, inc_t cst, ref double q, inc_t rsq, inc_t csq);

    // Tridiagonaling.Tridiag(A, T, d, e) (DDLA/Transformations/Tridiagonaling.cs:33-56): A <- Q
    [DllImport(Lib, EntryPoint = "ddla_dsytrd")]
    public static extern int SyTRD(dim_t n, ref double a, inc_t rsa, inc_t csa, ref double t, dim_t tRows,
        inc_t rst, inc_t cst, ref double d, ref double e, in Opts opts);

    // Bidiagonaling.Bidiag2(A, U, V, d, e) (DDLA/Transformations/Bidiagonaling.cs:48-60), m >= n
    [DllImport(Lib, EntryPoint = "ddla_dbidiag")]
    public static extern int Bidiag2(dim_t m, dim_t n, ref double a, inc_t rsa, inc_t csa, ref double d, ref double e,
        ref double u, inc_t rsu, inc_t csu, ref double v, inc_t rsv, inc_t csv, in Opts opts);

    // Bidiagonaling.Bidiag(A, U, V, d, e) through TwoStageBidiag (Bidiagonaling.cs:24-32, 334-582), m >= n;
    // a is overwritten (pass a clone: DDLA's Bidiag leaves A unchanged)
    [DllImport(Lib, EntryPoint = "ddla_dbidiag_twostage")]
    public static extern int Bidiag(dim_t m, dim_t n, ref double a, inc_t rsa, inc_t csa, ref double d, ref double e,
        ref double u, inc_t rsu, inc_t csu, ref double v, inc_t rsv, inc_t csv, in Opts opts);

    // ------------------------------------------------------------ einsum

    /// <summary>ddla_contract_mode: length and element strides in A, B, C.</summary>
    [StructLayout(LayoutKind.Sequential)]
    public struct ContractMode { public long Len, Sa, Sb, Sc; }

    /// <summary>ddla_contract_desc, the lowered contraction (MArray.Contract's index analysis).</summary>
    [StructLayout(LayoutKind.Sequential)]
    public struct ContractDesc
    {
        public int NBatch, NM, NN, NK, Swapped, Reserved;
        [MarshalAs(UnmanagedType.ByValArray, SizeConst = 48)] public ContractMode[] Batch;
        [MarshalAs(UnmanagedType.ByValArray, SizeConst = 16)] public ContractMode[] M;
        [MarshalAs(UnmanagedType.ByValArray, SizeConst = 16)] public ContractMode[] N;
        [MarshalAs(UnmanagedType.ByValArray, SizeConst = 16)] public ContractMode[] K;
    }

    // MArray.Contract's index analysis (DDLA/Einsum/MArray.Contract.cs:48-125)
    [DllImport(Lib, EntryPoint = "ddla_contract_plan")]
    public static extern int ContractPlan(string expr, int rankA, long[] lenA, long[] strA, int rankB, long[] lenB,
        long[] strB, int rankC, long[] lenC, long[] strC, out ContractDesc desc);
    // C += alpha * contraction(A, B); a / b / c point at the element with all indices 0
    [DllImport(Lib, EntryPoint = "ddla_contract")]
    public static extern int Contract(in ContractDesc desc, double alpha, ref double a, long na, ref double b, long nb,
        ref double c, long nc, int precision);
    // MArray.Einsum (MArray.Contract.cs:409-427): lens / strides / inputs are arrays of pointers
    [DllImport(Lib, EntryPoint = "ddla_einsum")]
    public static extern int Einsum(string expr, int nInputs, int[] ranks, IntPtr[] lens, IntPtr[] strides,
        IntPtr[] inputs, long[] counts, double alpha, double beta, int rankOut, long[] lenOut, long[] strOut,
        ref double output, long outCount, int precision);
    [DllImport(Lib, EntryPoint = "ddla_einsum_path")]
    public static extern int EinsumPath(string expr, int nInputs, int[] ranks, IntPtr[] lens, byte[] buf, int buflen);

    // ------------------------------------------------------------ status -> DDLA's exceptions

    /// <summary>0 passes; a positive status is DDLA's LinalgException (failing pivot), a
    /// small negative one its ArgumentException, the rest a runtime failure.</summary>
    public static void Check(int rc, string what)
    {
        if (rc == 0) return;
        if (rc > 0) throw new LinalgException(what, rc, $"failing pivot at index {rc - 1}");
        if (rc > -1000) throw new ArgumentException($"{what}: argument {-rc}: {LastError()}");
        throw new InvalidOperationException($"{what}: {LastError()}");
    }
}
