"""TypeParameter (hoomd/data/typeparam.py): a named type parameter of an operation, added with
the operation's ``_add_typeparam``; the operation then exposes it as the attribute ``name``."""


class TypeParameter:
    def __init__(self, name, type_kind, param_dict):
        self.name = name
        self.type_kind = type_kind
        self.param_dict = param_dict

    def make_container(self):
        return self.param_dict.make_container()
