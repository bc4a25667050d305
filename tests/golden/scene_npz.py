"""Save / load a SceneData plus its render settings as one .npz (arrays plus a
JSON header), the form in which the reference's glTF test fixtures are
committed (the GPU machine has no copy of the reference)."""
import json

import numpy as np

from mitrace_gb300.scenes import (CameraData, InstanceData, LightData, MaterialData, MeshData, SceneData,
                                  TextureData, config_dict, make_config)


def save_scene(path, scene: SceneData, cfg, meta=None):
    arrays, head = {}, {"meshes": [], "instances": [], "materials": [], "textures": [], "lights": [],
                        "camera": {}, "config": config_dict(cfg), "meta": meta or {}}
    for i, m in enumerate(scene.meshes):
        arrays[f"m{i}_pos"] = m.positions
        arrays[f"m{i}_nrm"] = m.normals
        if m.uv0 is not None:
            arrays[f"m{i}_uv"] = m.uv0
        head["meshes"].append({"uv": m.uv0 is not None})
    for x in scene.instances:
        head["instances"].append({"mesh": x.mesh, "material": x.material})
    arrays["inst_xf"] = np.stack([x.transform for x in scene.instances]).astype(np.float32)
    for mt in scene.materials:
        head["materials"].append(mt.__dict__.copy())
    for i, t in enumerate(scene.textures):
        if t.rgb8 is not None:
            arrays[f"t{i}"] = t.rgb8
        else:
            arrays[f"t{i}"] = t.rgb32f
        head["textures"].append({"filter": t.filter, "offset": list(t.offset), "scale": list(t.scale)})
    for L in scene.lights:
        head["lights"].append({k: (list(v) if isinstance(v, tuple) else v) for k, v in L.__dict__.items()})
    c = scene.camera
    head["camera"] = {"type": c.type, "yfov": c.yfov, "aspect": c.aspect, "ortho": list(c.ortho)}
    arrays["cam_xf"] = np.asarray(c.cam_to_world, np.float32)
    head["env"] = scene.env
    arrays["header"] = np.frombuffer(json.dumps(head).encode(), np.uint8)
    np.savez_compressed(path, **arrays)


def load_scene(path):
    z = np.load(path)
    head = json.loads(bytes(z["header"]).decode())
    meshes = [MeshData(positions=z[f"m{i}_pos"], normals=z[f"m{i}_nrm"], uv0=z[f"m{i}_uv"] if m["uv"] else None)
              for i, m in enumerate(head["meshes"])]
    xf = z["inst_xf"]
    inst = [InstanceData(mesh=d["mesh"], material=d["material"], transform=xf[k].copy())
            for k, d in enumerate(head["instances"])]
    mats = []
    for d in head["materials"]:
        d = {k: (tuple(v) if isinstance(v, list) else v) for k, v in d.items()}
        mats.append(MaterialData(**d))
    texs = []
    for i, d in enumerate(head["textures"]):
        a = z[f"t{i}"]
        kw = {"rgb8": a} if a.dtype == np.uint8 else {"rgb32f": a}
        texs.append(TextureData(filter=d["filter"], offset=tuple(d["offset"]), scale=tuple(d["scale"]), **kw))
    lights = [LightData(**{k: (tuple(v) if isinstance(v, list) else v) for k, v in d.items()}) for d in head["lights"]]
    c = head["camera"]
    cam = CameraData(type=c["type"], cam_to_world=z["cam_xf"].copy(), yfov=c["yfov"], aspect=c["aspect"],
                     ortho=tuple(c["ortho"]))
    scene = SceneData(meshes=meshes, instances=inst, materials=mats, textures=texs, lights=lights, camera=cam,
                      env=head["env"])
    cfg = make_config(**{k: v for k, v in head["config"].items()})
    return scene, cfg, head["meta"]
