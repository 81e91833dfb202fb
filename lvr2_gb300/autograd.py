"""torch.autograd binding of the signed distance of AdaptiveKSearchSurface
(AdaptiveKSearchSurface.tcc:414-457) through lvrgb_distance_adjoint.

    d, e = signed_distance(surface, q, points, normals)

returns the projected and Euclidean distances of the CUDA tensor q (n, 3);
their backward gives gradients with respect to q and, when `points` /
`normals` are tensors that require grad, with respect to the surface's points
and normals (the tensors the surface was built from and set with
set_normals, in the same order).  Each query's kd nearest points are held
fixed, as the distance is piecewise smooth in q.
"""
import torch


class SignedDistance(torch.autograd.Function):
    @staticmethod
    def forward(ctx, surface, queries, points, normals):
        q = queries.detach().contiguous()
        proj, eucl, _, _, _ = surface.distance_adjoint(q, want_points=False, want_normals=False)
        ctx.surface = surface
        ctx.save_for_backward(q)
        return proj, eucl

    @staticmethod
    def backward(ctx, grad_proj, grad_eucl):
        (q,) = ctx.saved_tensors
        need_p = ctx.needs_input_grad[2]
        need_n = ctx.needs_input_grad[3]
        gd = None if grad_proj is None else grad_proj.contiguous()
        ge = None if grad_eucl is None else grad_eucl.contiguous()
        _, _, gq, gp, gn = ctx.surface.distance_adjoint(q, gd, ge, want_points=need_p, want_normals=need_n)
        return None, (gq if ctx.needs_input_grad[1] else None), gp, gn


def signed_distance(surface, queries, points=None, normals=None):
    """Differentiable (projected, euclidean) distance of `queries` to `surface`."""
    return SignedDistance.apply(surface, queries, points, normals)
