// The provider switch: DDLA's factorization entry points with the GPU library
// behind them, same signatures and conventions.
//
// DDLA's LU / Cholesky / LDLT static methods (DDLA/Factorizations/LU.cs:133-287,
// Cholesky.cs:52-123, LDLT.cs:56-126) call this class first when
// CudaProvider.UseCuda is set (one line at the top of each method):
//
//     public static void PLUDecompose(MatrixView A, Span<int> pivs)
//     {
//         if (CudaProvider.UseCuda) { CudaProvider.PLUDecompose(A, pivs); return; }
//         ...
//
// and BlasProvider's checked level-3 wrappers (DDLA/BLAS/3m.cs:10-305) do the
// same through the BLIS-shaped calls.  Every call is synchronous: the results
// are in the caller's arrays when it returns.
using System;
using DDLA.Core;
using DDLA.Misc.Flags;

namespace DDLA.BLAS.Cuda;

public static class CudaProvider
{
    /// <summary>Route DDLA's factorizations and level-3 calls to libddla_gb300.</summary>
    public static bool UseCuda { get; set; }

    /// <summary>Options for every call (zero = library defaults; Precision = 4 runs the FP64
    /// factorizations' trailing updates through the split-precision tensor-core GEMM).</summary>
    public static Source.Opts Options = new();

    static void Square(MatrixView A)
    {
        if (A.Rows != A.Cols) throw new ArgumentException("Matrix must be square for LU factorization.");
    }

    // LU.PLUDecompose (LU.cs:251-264): pivots relative, row i <-> row i + pivs[i]
    public static void PLUDecompose(MatrixView A, Span<int> pivs)
    {
        Square(A);
        if (pivs.Length != A.Rows) throw new ArgumentException("Pivot array length must match matrix size.");
        if (A.Rows == 0) return;
        Source.Check(Source.GetRF(A.Rows, ref A.GetHeadRef(), A.RowStride, A.ColStride, ref pivs[0], in Options),
            "PLUDecompose");
    }

    // LU.PLUSolve (LU.cs:266-275)
    public static void PLUSolve(MatrixView A, Span<int> pivs, MatrixView B, bool trans = false)
    {
        Square(A);
        if (A.Rows != B.Rows) throw new ArgumentException("RHS matrix size mismatch", nameof(B));
        if (A.Rows == 0 || B.Cols == 0) return;
        Source.Check(Source.GetRS(trans ? 1 : 0, A.Rows, B.Cols, ref A.GetHeadRef(), A.RowStride, A.ColStride,
            ref pivs[0], ref B.GetHeadRef(), B.RowStride, B.ColStride), "PLUSolve");
    }

    // LU.LUDecompose / LUSolve (LU.cs:133-167)
    public static void LUDecompose(MatrixView A)
    {
        Square(A);
        if (A.Rows == 0) return;
        Source.Check(Source.GetRFNoPiv(A.Rows, ref A.GetHeadRef(), A.RowStride, A.ColStride, in Options),
            "LUDecompose");
    }

    public static void LUSolve(MatrixView A, MatrixView B, bool trans = false)
    {
        Square(A);
        if (A.Rows != B.Rows) throw new ArgumentException("RHS matrix size mismatch", nameof(B));
        if (A.Rows == 0 || B.Cols == 0) return;
        Source.Check(Source.GetRSNoPiv(trans ? 1 : 0, A.Rows, B.Cols, ref A.GetHeadRef(), A.RowStride, A.ColStride,
            ref B.GetHeadRef(), B.RowStride, B.ColStride), "LUSolve");
    }

    // Cholesky.CholDecompose / CholeskySolve (Cholesky.cs:52-123)
    public static void CholDecompose(UpLo uplo, MatrixView A)
    {
        Square(A);
        if (A.Rows == 0) return;
        Source.Check(Source.PotRF(uplo, A.Rows, ref A.GetHeadRef(), A.RowStride, A.ColStride, in Options),
            "CholDecompose");
    }

    public static void CholeskySolve(UpLo uplo, MatrixView A, MatrixView B)
    {
        Square(A);
        if (A.Rows != B.Rows) throw new ArgumentException("Matrix dimensions do not match for Cholesky solve.");
        if (A.Rows == 0 || B.Cols == 0) return;
        Source.Check(Source.PotRS(uplo, A.Rows, B.Cols, ref A.GetHeadRef(), A.RowStride, A.ColStride,
            ref B.GetHeadRef(), B.RowStride, B.ColStride), "CholeskySolve");
    }

    // LDLT.LDLTDecompose / LDLTSolve (LDLT.cs:56-126)
    public static void LDLTDecompose(UpLo uplo, MatrixView A)
    {
        Square(A);
        if (A.Rows == 0) return;
        Source.Check(Source.LDLT(uplo, A.Rows, ref A.GetHeadRef(), A.RowStride, A.ColStride, in Options),
            "LDLTDecompose");
    }

    public static void LDLTSolve(UpLo uplo, MatrixView A, MatrixView B)
    {
        Square(A);
        if (A.Rows != B.Rows) throw new ArgumentException("Matrix dimensions do not match for LDLT solve.");
        if (A.Rows == 0 || B.Cols == 0) return;
        Source.Check(Source.LDLTS(uplo, A.Rows, B.Cols, ref A.GetHeadRef(), A.RowStride, A.ColStride,
            ref B.GetHeadRef(), B.RowStride, B.ColStride), "LDLTSolve");
    }

    /// <summary>Mixed-precision solve of A X = B (FP32 factor, FP64 refinement to
    /// Options.Tol, default 1e-14); A and B unchanged.  kind: 0 LU, 1 Cholesky, 2 LDL^T.</summary>
    public static Source.SolveReport SolveMixed(MatrixView A, MatrixView B, MatrixView X, int kind = 0,
        UpLo uplo = UpLo.Lower)
    {
        Square(A);
        if (A.Rows != B.Rows || X.Rows != B.Rows || X.Cols != B.Cols)
            throw new ArgumentException("Matrix dimensions do not match for the solve.");
        Source.SolveReport rep;
        int rc = kind switch
        {
            0 => Source.GeSVMixed(A.Rows, B.Cols, ref A.GetHeadRef(), A.RowStride, A.ColStride, ref B.GetHeadRef(),
                B.RowStride, B.ColStride, ref X.GetHeadRef(), X.RowStride, X.ColStride, IntPtr.Zero, in Options,
                out rep),
            1 => Source.PoSVMixed(uplo, A.Rows, B.Cols, ref A.GetHeadRef(), A.RowStride, A.ColStride,
                ref B.GetHeadRef(), B.RowStride, B.ColStride, ref X.GetHeadRef(), X.RowStride, X.ColStride,
                IntPtr.Zero, in Options, out rep),
            _ => Source.SySVMixed(uplo, A.Rows, B.Cols, ref A.GetHeadRef(), A.RowStride, A.ColStride,
                ref B.GetHeadRef(), B.RowStride, B.ColStride, ref X.GetHeadRef(), X.RowStride, X.ColStride,
                IntPtr.Zero, in Options, out rep),
        };
        Source.Check(rc, "SolveMixed");
        return rep;
    }

    // Bidiagonaling.Bidiag(A, U, V, d, e) (DDLA/Transformations/Bidiagonaling.cs:24-32): the two-stage
    // reduction on a column-major clone of A, as TwoStageBidiag works (Bidiagonaling.cs:250-257)
    public static void Bidiag(MatrixView A, MatrixView U, MatrixView V, VectorView d, VectorView e)
    {
        if (A.Rows < A.Cols) throw new ArgumentException("Only support m >= n");
        if (A.Cols == 0) return;
        var W = A.Clone(colMajor: true);
        var dd = VectorView.Create(A.Cols);
        var ee = VectorView.Create(Math.Max(A.Cols - 1, 1));
        Source.Check(Source.Bidiag(A.Rows, A.Cols, ref W.GetHeadRef(), W.RowStride, W.ColStride, ref dd.GetHeadRef(),
            ref ee.GetHeadRef(), ref U.GetHeadRef(), U.RowStride, U.ColStride, ref V.GetHeadRef(), V.RowStride,
            V.ColStride, in Options), "Bidiag");
        dd.CopyTo(d);
        if (A.Cols > 1) ee[..(A.Cols - 1)].CopyTo(e);
    }

    // BlasProvider.GeMM's checked wrapper (DDLA/BLAS/3m.cs:10-31) on the GPU
    public static void GeMM(double alpha, MatrixView A, MatrixView B, double beta, MatrixView C)
    {
        if (A.Rows != C.Rows || B.Cols != C.Cols || A.Cols != B.Rows)
            throw new ArgumentException("Dimensions of matrix A must be match!");
        Source.Check(Source.GeMM(TransType.NoTrans, TransType.NoTrans, C.Rows, C.Cols, A.Cols, in alpha,
            ref A.GetHeadRef(), A.RowStride, A.ColStride, ref B.GetHeadRef(), B.RowStride, B.ColStride,
            in beta, ref C.GetHeadRef(), C.RowStride, C.ColStride), "GeMM");
    }
}
