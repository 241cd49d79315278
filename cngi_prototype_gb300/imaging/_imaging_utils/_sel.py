"""Data-group selection, as cngi/_utils/_check_parms.py:_check_sel_parms (:122-223).

A dataset's attrs['data_groups'][0] maps group ids to {'id', role -> variable
name}. The input group is sel_parms['data_group_in_id'] (default: the first
group); the output group copies it, adds the roles the function creates
(overridable by name in sel_parms) and keeps the input id when
append_to_in_id, otherwise takes the next free id (or data_group_out_id).
Input roles must name variables present in the dataset.
"""
import copy


def _check_sel_parms(xds, sel_parms, new_or_modified_data_variables=None, required_data_variables=None,
                     append_to_in_id=False):
    new = dict(new_or_modified_data_variables or {})
    req = dict(required_data_variables or {})
    if 'data_groups' not in xds.attrs:
        gid = str(sel_parms.get('data_group_out_id', '0'))
        xds.attrs['data_groups'] = [{gid: {'id': gid}}]
        append_to_in_id = True
    groups = xds.attrs['data_groups'][0]
    ids = [int(k) for k in groups]
    if 'data_group_in_id' in sel_parms:
        key = str(sel_parms['data_group_in_id'])
        if key not in groups:
            raise AssertionError(f'######### ERROR: data_group_in id {key} does not exist')
        gin = copy.deepcopy(groups[key])
    elif 'data_group_in' in sel_parms and isinstance(sel_parms['data_group_in'], dict):
        gin = copy.deepcopy(sel_parms['data_group_in'])
        gin.setdefault('id', '-1')
    else:
        gin = copy.deepcopy(next(iter(groups.values())))
    out_id = gin.get('id', '0') if append_to_in_id else str(max(ids) + 1)
    if 'data_group_out_id' in sel_parms:
        out_id = str(sel_parms['data_group_out_id'])
    gin = {**req, **gin}
    gout = {**gin, 'id': str(out_id), **new}
    for k in new:
        if k in sel_parms and isinstance(sel_parms[k], str):
            gout[k] = sel_parms[k]
    if isinstance(sel_parms.get('data_group_out'), dict):
        for k, v in sel_parms['data_group_out'].items():
            if k in new or k == 'id':
                gout[k] = v
    for role, name in gin.items():
        if role in ('id', 'properties'):
            continue
        if name not in xds:
            raise AssertionError(f'######### ERROR Data array {name} can not be found in dataset.')
    sel_parms['data_group_in'] = gin
    sel_parms['data_group_out'] = gout
    return True


def _register_group(xds, gout):
    groups = xds.attrs['data_groups'][0]
    groups[str(gout['id'])] = {**groups.get(str(gout['id']), {}), **gout}
