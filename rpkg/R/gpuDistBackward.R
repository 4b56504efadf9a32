# Gradient of the euclidean gpuDist(points) with respect to the points.
# No counterpart in the reference: it is the adjoint of R/gpuHclust.R's
# gpuDist(method = "euclidean"), computed on the GPU by RgpuDistBackward.
#   points  n x d numeric matrix, one point per row, as for gpuDist(points)
#   grad    n x n matrix dL/dD of a scalar loss L of D = as.matrix(gpuDist(points));
#           both triangles count, pairs at distance 0 contribute nothing
# Returns the n x d matrix dL/dpoints.
gpuDistBackward <- function(points, grad) {
    points <- as.matrix(points)
    n <- nrow(points)
    d <- ncol(points)
    grad <- as.matrix(grad)
    if(nrow(grad) != n || ncol(grad) != n) {
        stop("grad must be a nrow(points) by nrow(points) matrix")
    }
    dx <- .C("RgpuDistBackward",
             as.single(t(points)), as.integer(n), as.integer(d),
             as.single(t(grad)), dx = single(n * d),
             PACKAGE='gputools')$dx
    t(matrix(as.double(dx), d, n, dimnames = rev(dimnames(points))))
}
