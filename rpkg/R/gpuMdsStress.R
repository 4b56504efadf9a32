# Metric MDS stress sum_{i<j} (D_ij - delta_ij)^2 of a point configuration
# against target dissimilarities, with its gradient, on the GPU
# (RgpuMdsStress).  No counterpart in the reference: it is the loss
# gpuDistBackward differentiates, fused so that the n x n distances never
# leave the device.
#   points  n x d numeric matrix, one point per row
#   delta   a dist object (or a vector in dist order) of the n targets
# Returns list(stress, gradient) with gradient the n x d matrix dstress/dpoints.
gpuMdsStress <- function(points, delta) {
    points <- as.matrix(points)
    n <- nrow(points)
    d <- ncol(points)
    delta <- as.vector(delta)
    if(length(delta) != n * (n - 1) / 2) {
        stop("delta must hold n * (n - 1) / 2 dissimilarities (a dist object)")
    }
    r <- .C("RgpuMdsStress",
            as.single(t(points)), as.integer(n), as.integer(d),
            as.single(delta), loss = double(1), dx = single(n * d),
            PACKAGE='gputools')
    list(stress = r$loss,
         gradient = t(matrix(as.double(r$dx), d, n, dimnames = rev(dimnames(points)))))
}
