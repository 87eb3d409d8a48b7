"""Depth and blend states that together exercise every VkCompareOp, every single-source VkBlendFactor in each
of the four factor slots, every VkBlendOp in both op slots, blend constants (inside and outside [0, 1]) and
partial colour write masks.  Shared by the oracle's CPU tests and the GPU parity tests."""

COMPARE_OPS = {0: "never", 1: "less", 2: "equal", 3: "lequal", 4: "greater", 5: "notequal", 6: "gequal", 7: "always"}

# clear depth per compare op that lets the op pass for some fragments of the test scenes (depths in (0, 1))
CLEAR_DEPTH = {0: 1.0, 1: 1.0, 2: 0.25, 3: 1.0, 4: 0.0, 5: 1.0, 6: 0.0, 7: 0.5}

N_FACTORS = 15  # VK_BLEND_FACTOR_ZERO .. VK_BLEND_FACTOR_SRC_ALPHA_SATURATE
N_OPS = 5       # VK_BLEND_OP_ADD .. VK_BLEND_OP_MAX


def blend_states():
    """15 blend states (srcColor, dstColor, colorOp, srcAlpha, dstAlpha, alphaOp): state i puts factor i in the
    source colour slot, and a rotation of the factors in the other three, so that every factor appears in every
    slot; the ops cycle so that each op appears in both op slots"""
    out = []
    for i in range(N_FACTORS):
        out.append((i, (i + 5) % N_FACTORS, i % N_OPS, (i + 3) % N_FACTORS, (i + 11) % N_FACTORS, (i + 2) % N_OPS))
    return out


# blend constants per state (cycled): some outside [0, 1], which the attachment's normalized range clamps
BLEND_CONSTS = [(0.25, 0.5, 0.75, 0.6), (1.5, -0.25, 0.3, 0.9), (0.0, 1.0, 0.125, 0.0), (0.8, 0.2, 2.0, -1.0)]
# colour write masks per state (cycled)
WRITE_MASKS = [0xF, 0x7, 0xA, 0x5, 0x1, 0xE, 0x0, 0x8]
