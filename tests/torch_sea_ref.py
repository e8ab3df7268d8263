"""Plain-PyTorch FP64 restatement of the reference's se_e2_a descriptor for
the GPU tests: the environment matrix of deepmd/pt/model/descriptor/
env_mat.py:18-119 and the block of deepmd/pt/model/descriptor/se_a.py:742-858,
written with differentiable torch ops so that torch.autograd gives the first
and second derivatives the dpgb kernels are checked against.  Test
infrastructure only."""
import torch


def smooth_weight(r, rmin, rmax):
    # deepmd/pt/utils/preprocess.py compute_smooth_weight
    r = torch.clamp(r, min=rmin, max=rmax)
    uu = (r - rmin) / (rmax - rmin)
    return uu * uu * uu * (-6 * uu * uu + 15 * uu - 10) + 1


def env_mat(coord_ext, nlist, atype, mean, stddev, rcut, rcut_smth, protection=0.0):
    nf, nloc, nnei = nlist.shape
    coord = coord_ext.view(nf, -1, 3)
    nall = coord.shape[1]
    mask = nlist >= 0
    nl = torch.where(mask, nlist, nall)
    centre = coord[:, :nloc].view(nf, -1, 1, 3)
    idx = nl.view(nf, -1).unsqueeze(-1).expand(-1, -1, 3)
    padded = torch.cat([coord, coord[:, -1:, :] + rcut], dim=1)
    nbr = torch.gather(padded, 1, idx).view(nf, nloc, nnei, 3)
    diff = nbr - centre
    length = torch.linalg.norm(diff, dim=-1, keepdim=True) + (~mask).unsqueeze(-1)
    t0 = 1 / (length + protection)
    t1 = diff / (length + protection) ** 2
    w = smooth_weight(length, rcut_smth, rcut) * mask.unsqueeze(-1)
    em = torch.cat([t0, t1], dim=-1) * w
    return (em - mean[atype]) / stddev[atype], diff * mask.unsqueeze(-1), w


def mlp(ss, layers, resnet_dt):
    x = ss
    for W, b, idt in layers:
        y = torch.tanh(torch.matmul(x, W) + b)
        if resnet_dt:
            y = y * idt
        if W.shape[1] == W.shape[0]:
            y = y + x
        elif W.shape[1] == 2 * W.shape[0]:
            y = y + torch.cat([x, x], dim=-1)
        x = y
    return x


def block(rr, nlist, atype_ext, nets, sel, type_one_side, resnet_dt, axis, keep=None):
    """rr [nf*nloc, nnei, 4]; nets[e] = [(W, b, idt), ...]; keep (ntypes+1)^2
    0/1 table or None -> (descriptor [nf*nloc, ng*M], xyz [nf*nloc, 4, ng])."""
    nf, nloc, nnei = nlist.shape
    ntypes = len(sel)
    sec = [0]
    for s in sel:
        sec.append(sec[-1] + s)
    atype = atype_ext[:, :nloc].reshape(-1)
    if keep is not None:
        nall = atype_ext.shape[1]
        ae = torch.cat([atype_ext, torch.full((nf, 1), ntypes, dtype=atype_ext.dtype, device=atype_ext.device)], 1)
        idx = torch.where(nlist < 0, torch.full_like(nlist, nall), nlist).view(nf, -1)
        tj = torch.gather(ae, 1, idx).view(nf * nloc, nnei)
        mask = keep.to(rr.device)[atype.view(-1, 1).long(), tj.long()].to(rr.dtype)
    else:
        mask = torch.ones(rr.shape[:2], dtype=rr.dtype, device=rr.device)
    ng = nets[0][-1][0].shape[1]
    xyz = torch.zeros((rr.shape[0], 4, ng), dtype=rr.dtype, device=rr.device)
    for e, layers in enumerate(nets):
        if type_one_side:
            ii, rows = e, None
        else:
            ii, ti = e // ntypes, e % ntypes
            rows = atype.eq(ti)
        r = rr[:, sec[ii]:sec[ii + 1], :] if rows is None else rr[rows, sec[ii]:sec[ii + 1], :]
        m = mask[:, sec[ii]:sec[ii + 1]] if rows is None else mask[rows, sec[ii]:sec[ii + 1]]
        r = r * m[:, :, None]
        gg = mlp(r[:, :, :1], layers, resnet_dt)
        gr = torch.matmul(r.permute(0, 2, 1), gg)
        if rows is None:
            xyz = xyz + gr
        else:
            xyz = xyz.index_put((rows.nonzero().squeeze(1),), gr, accumulate=True)
    xyz = xyz / nnei
    D = torch.matmul(xyz.permute(0, 2, 1), xyz[:, :, :axis]).reshape(rr.shape[0], -1)
    return D, xyz


def nets_from_flat(flat, ntypes, neuron, type_one_side, resnet_dt):
    """Split the kernels' flat parameter vector into per-net layer tuples."""
    nnets = ntypes if type_one_side else ntypes * ntypes
    widths = [1, *neuron]
    nets, off = [], 0
    for _ in range(nnets):
        layers = []
        for l in range(len(neuron)):
            nin, nout = widths[l], widths[l + 1]
            W = flat[off:off + nin * nout].view(nin, nout)
            off += nin * nout
            b = flat[off:off + nout]
            off += nout
            idt = None
            if resnet_dt:
                idt = flat[off:off + nout]
                off += nout
            layers.append((W, b, idt))
        nets.append(layers)
    assert off == flat.numel()
    return nets
