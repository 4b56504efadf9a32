# Gradient of gpuCor(x) (Pearson, use = "everything") with respect to x.
# No counterpart in the reference: it is the adjoint of R/gpuCor.R's
# coefficient matrix, computed on the GPU by RgpuCorBackward (means and norms
# recomputed, the contraction on the tensor cores).
#   x     n x p numeric matrix (observations in rows), as for gpuCor(x)
#   grad  p x p matrix dL/dC of a scalar loss L of C = gpuCor(x)$coefficients
# Returns the n x p matrix dL/dx; a constant column gets a zero gradient.
gpuCorBackward <- function(x, grad) {
    x <- as.matrix(x)
    n <- nrow(x)
    p <- ncol(x)
    grad <- as.matrix(grad)
    if(nrow(grad) != p || ncol(grad) != p) {
        stop("grad must be a ncol(x) by ncol(x) matrix")
    }
    dx <- .C("RgpuCorBackward",
             as.single(x), as.integer(n), as.integer(p),
             as.single(grad), dx = single(n * p),
             PACKAGE='gputools')$dx
    matrix(as.double(dx), n, p, dimnames = dimnames(x))
}
